// Kernel instantiations for dtype f32, nx = 5 (all compiled ny).
#include "ss_run.cuh"

SS_INST(float, f32, 5, 1)
SS_INST(float, f32, 5, 2)
SS_INST(float, f32, 5, 3)
