// Kernel instantiations for dtype f32, nx = 2 (all compiled ny).
#include "ss_run.cuh"

SS_INST(float, f32, 2, 1)
SS_INST(float, f32, 2, 2)
SS_INST(float, f32, 2, 3)
