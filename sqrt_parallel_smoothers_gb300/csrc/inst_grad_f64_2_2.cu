// Forward-mode gradient instantiations for dtype f64, (nx, ny) = (2, 2).
#include "ss_grad.cuh"

SS_INST_GRAD(double, f64, 2, 2)
