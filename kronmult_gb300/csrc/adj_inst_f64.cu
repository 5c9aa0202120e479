// Explicit instantiation of the adjoint kernels for double.
#include "adj_kernels.cuh"
KGB_ADJ_INSTANTIATE(double)
