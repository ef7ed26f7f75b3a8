// Kernel instantiations for dtype f64, (nx, ny) = (7, 2).
#include "ss_run.cuh"

SS_INST(double, f64, 7, 2)
