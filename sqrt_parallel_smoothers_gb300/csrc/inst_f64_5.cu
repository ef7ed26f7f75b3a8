// Kernel instantiations for dtype f64, nx = 5 (all compiled ny).
#include "ss_run.cuh"

SS_INST(double, f64, 5, 1)
SS_INST(double, f64, 5, 2)
SS_INST(double, f64, 5, 3)
