// Forward-mode gradient instantiations for dtype f32, (nx, ny) = (5, 2).
#include "ss_grad.cuh"

SS_INST_GRAD(float, f32, 5, 2)
