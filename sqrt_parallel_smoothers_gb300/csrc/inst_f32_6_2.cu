// Kernel instantiations for dtype f32, (nx, ny) = (6, 2).
#include "ss_run.cuh"

SS_INST(float, f32, 6, 2)
