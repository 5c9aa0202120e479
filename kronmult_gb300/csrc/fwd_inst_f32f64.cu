// Explicit instantiation of the forward kernels for (storage, output) = (float,double).
#include "fwd_kernels.cuh"
#include "split_kernels.cuh"
KGB_FWD_INSTANTIATE(float, double)
KGB_SPLIT_INSTANTIATE(float, double)
