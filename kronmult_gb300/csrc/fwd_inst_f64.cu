// Explicit instantiation of the forward kernels for (storage, output) = (double,double).
#include "fwd_kernels.cuh"
#include "split_kernels.cuh"
KGB_FWD_INSTANTIATE(double, double)
KGB_SPLIT_NONE(double, double)
