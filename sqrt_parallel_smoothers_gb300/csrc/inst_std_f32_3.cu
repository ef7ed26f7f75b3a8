// Covariance-form kernel instantiations for dtype f32, nx = 3 (ny = 1, 2, 3).
#include "ss_std_run.cuh"

SS_INST_STD(float, 3, 1)
SS_INST_STD(float, 3, 2)
SS_INST_STD(float, 3, 3)
