// Transposed (vector-Jacobian) forward step of the reversible gradient.
#pragma once
#include "fdtd_kernels.cuh"
