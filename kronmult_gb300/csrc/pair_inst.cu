// Explicit instantiation of the two-modes-per-pass FP32 forward (outputs FP32 and FP64).
#include "pair_kernels.cuh"
KGB_PAIR_INSTANTIATE(float)
KGB_PAIR_INSTANTIATE(double)
