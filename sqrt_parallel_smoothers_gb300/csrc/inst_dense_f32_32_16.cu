// Dense-path kernel instantiations for dtype f32, (nx, ny) = (32, 16).
#include "ss_dense_run.cuh"

SS_INST_DENSE(float, f32, 32, 16)
