// Kernel instantiations for dtype f32, nx = 1 (all compiled ny).
#include "ss_run.cuh"

SS_INST(float, f32, 1, 1)
SS_INST(float, f32, 1, 2)
SS_INST(float, f32, 1, 3)
