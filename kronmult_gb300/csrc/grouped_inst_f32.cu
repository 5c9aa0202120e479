// Explicit instantiation of the grouped forward's FP32 kernels.
#include "grouped_kernels.cuh"
#define KGB_T float
#define KGB_TO float
namespace kgb {
KGB_GQ_LOOKUP_FIBRE_AND_RT
KGB_GQ_LOOKUP_NO_ELEM
}  // namespace kgb
