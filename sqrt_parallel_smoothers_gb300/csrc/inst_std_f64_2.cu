// Covariance-form kernel instantiations for dtype f64, nx = 2 (ny = 1, 2, 3).
#include "ss_std_run.cuh"

SS_INST_STD(double, 2, 1)
SS_INST_STD(double, 2, 2)
SS_INST_STD(double, 2, 3)
