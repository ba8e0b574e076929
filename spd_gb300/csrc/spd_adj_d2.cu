// Adjoint launch sequences for 2D (p = 1..4).
#include "spd_adjoint_exec.cuh"

SPD_INSTANTIATE_ADJOINT(2)
