// Kernel instantiations for dtype f64, nx = 4 (all compiled ny).
#include "ss_run.cuh"

SS_INST(double, f64, 4, 1)
SS_INST(double, f64, 4, 2)
SS_INST(double, f64, 4, 3)
