// Kernel instantiations for dtype f32, (nx, ny) = (3, 2).
#include "ss_run.cuh"

SS_INST(float, f32, 3, 2)
