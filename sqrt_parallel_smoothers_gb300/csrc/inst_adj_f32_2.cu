// Reverse-mode gradient instantiations for dtype f32, nx = 2, ny = 1..3.
#include "ss_adjoint.cuh"

SS_INST_ADJ(float, f32, 2, 1)
SS_INST_ADJ(float, f32, 2, 2)
SS_INST_ADJ(float, f32, 2, 3)
