// Kernel instantiations for dtype f32, (nx, ny) = (1, 3).
#include "ss_run.cuh"

SS_INST(float, f32, 1, 3)
