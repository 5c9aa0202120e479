// Explicit instantiation of the forward kernels for (storage, output) = (float,float).
#include "fwd_kernels.cuh"
#include "split_kernels.cuh"
KGB_FWD_INSTANTIATE(float, float)
KGB_SPLIT_INSTANTIATE(float, float)
