// Dense-path kernel instantiations for dtype f64, (nx, ny) = (32, 16).
#include "ss_dense_run.cuh"

SS_INST_DENSE(double, f64, 32, 16)
