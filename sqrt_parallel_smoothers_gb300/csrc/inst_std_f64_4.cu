// Covariance-form kernel instantiations for dtype f64, nx = 4 (ny = 1, 2, 3).
#include "ss_std_run.cuh"

SS_INST_STD(double, 4, 1)
SS_INST_STD(double, 4, 2)
SS_INST_STD(double, 4, 3)
