// Kernel instantiations for dtype f32, (nx, ny) = (7, 1).
#include "ss_run.cuh"

SS_INST(float, f32, 7, 1)
