// Kernel instantiations for dtype f32, (nx, ny) = (3, 3).
#include "ss_run.cuh"

SS_INST(float, f32, 3, 3)
