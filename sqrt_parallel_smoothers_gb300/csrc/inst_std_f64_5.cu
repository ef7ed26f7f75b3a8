// Covariance-form kernel instantiations for dtype f64, nx = 5 (ny = 1, 2, 3).
#include "ss_std_run.cuh"

SS_INST_STD(double, 5, 1)
SS_INST_STD(double, 5, 2)
SS_INST_STD(double, 5, 3)
