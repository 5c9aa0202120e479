// Explicit instantiation of the adjoint kernels for float.
#include "adj_kernels.cuh"
KGB_ADJ_INSTANTIATE(float)
KGB_ADJ_FIBRE_INSTANTIATE(float)
