// Dense-path kernel instantiations for dtype f32, (nx, ny) = (8, 4).
#include "ss_dense_run.cuh"

SS_INST_DENSE(float, f32, 8, 4)
