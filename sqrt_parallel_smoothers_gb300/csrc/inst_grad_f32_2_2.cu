// Forward-mode gradient instantiations for dtype f32, (nx, ny) = (2, 2).
#include "ss_grad.cuh"

SS_INST_GRAD(float, f32, 2, 2)
