// Kernel instantiations for dtype f64, (nx, ny) = (6, 1).
#include "ss_run.cuh"

SS_INST(double, f64, 6, 1)
