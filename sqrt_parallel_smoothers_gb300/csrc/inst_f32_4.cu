// Kernel instantiations for dtype f32, nx = 4 (all compiled ny).
#include "ss_run.cuh"

SS_INST(float, f32, 4, 1)
SS_INST(float, f32, 4, 2)
SS_INST(float, f32, 4, 3)
