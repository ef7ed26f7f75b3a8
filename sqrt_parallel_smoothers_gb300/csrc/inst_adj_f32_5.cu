// Reverse-mode gradient instantiations for dtype f32, nx = 5, ny = 1..3.
#include "ss_adjoint.cuh"

SS_INST_ADJ(float, f32, 5, 1)
SS_INST_ADJ(float, f32, 5, 2)
SS_INST_ADJ(float, f32, 5, 3)
