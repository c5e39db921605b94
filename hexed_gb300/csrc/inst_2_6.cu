// Kernels and launch sequences for n_dim 2, row size 6 (one unit per row size so they compile in parallel).
#include "ops.cuh"
HEXED_INSTANTIATE(2, 6)
