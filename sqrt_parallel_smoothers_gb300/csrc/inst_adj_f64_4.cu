// Reverse-mode gradient instantiations for dtype f64, nx = 4, ny = 1..3.
#include "ss_adjoint.cuh"

SS_INST_ADJ(double, f64, 4, 1)
SS_INST_ADJ(double, f64, 4, 2)
SS_INST_ADJ(double, f64, 4, 3)
