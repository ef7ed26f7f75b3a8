// Kernel instantiations for dtype f64, nx = 1 (all compiled ny).
#include "ss_run.cuh"

SS_INST(double, f64, 1, 1)
SS_INST(double, f64, 1, 2)
SS_INST(double, f64, 1, 3)
