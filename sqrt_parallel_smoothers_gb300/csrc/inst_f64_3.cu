// Kernel instantiations for dtype f64, nx = 3 (all compiled ny).
#include "ss_run.cuh"

SS_INST(double, f64, 3, 1)
SS_INST(double, f64, 3, 2)
SS_INST(double, f64, 3, 3)
