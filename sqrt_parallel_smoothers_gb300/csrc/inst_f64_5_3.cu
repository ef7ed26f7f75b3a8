// Kernel instantiations for dtype f64, (nx, ny) = (5, 3).
#include "ss_run.cuh"

SS_INST(double, f64, 5, 3)
