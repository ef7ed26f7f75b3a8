// Reverse-mode gradient instantiations for dtype f64, nx = 1, ny = 1..3.
#include "ss_adjoint.cuh"

SS_INST_ADJ(double, f64, 1, 1)
SS_INST_ADJ(double, f64, 1, 2)
SS_INST_ADJ(double, f64, 1, 3)
