// Reverse-mode gradient instantiations for dtype f64, nx = 3, ny = 1..3.
#include "ss_adjoint.cuh"

SS_INST_ADJ(double, f64, 3, 1)
SS_INST_ADJ(double, f64, 3, 2)
SS_INST_ADJ(double, f64, 3, 3)
