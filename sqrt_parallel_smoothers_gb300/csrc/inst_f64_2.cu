// Kernel instantiations for dtype f64, nx = 2 (all compiled ny).
#include "ss_run.cuh"

SS_INST(double, f64, 2, 1)
SS_INST(double, f64, 2, 2)
SS_INST(double, f64, 2, 3)
