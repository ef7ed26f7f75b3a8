// Kernel instantiations for dtype f32, nx = 3 (all compiled ny).
#include "ss_run.cuh"

SS_INST(float, f32, 3, 1)
SS_INST(float, f32, 3, 2)
SS_INST(float, f32, 3, 3)
