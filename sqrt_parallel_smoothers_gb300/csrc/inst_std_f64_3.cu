// Covariance-form kernel instantiations for dtype f64, nx = 3 (ny = 1, 2, 3).
#include "ss_std_run.cuh"

SS_INST_STD(double, 3, 1)
SS_INST_STD(double, 3, 2)
SS_INST_STD(double, 3, 3)
