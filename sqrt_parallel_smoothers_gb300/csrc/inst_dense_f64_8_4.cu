// Dense-path kernel instantiations for dtype f64, (nx, ny) = (8, 4).
#include "ss_dense_run.cuh"

SS_INST_DENSE(double, f64, 8, 4)
