// Kernels and launch sequences for n_dim 3, row size 2 (one unit per row size so they compile in parallel).
#include "ops.cuh"
HEXED_INSTANTIATE(3, 2)
