// Kernel instantiations for dtype f32, (nx, ny) = (4, 3).
#include "ss_run.cuh"

SS_INST(float, f32, 4, 3)
