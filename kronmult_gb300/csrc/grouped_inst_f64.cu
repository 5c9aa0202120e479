// Explicit instantiation of the grouped forward's FP64 kernels.
#include "grouped_kernels.cuh"
#define KGB_T double
#define KGB_TO double
namespace kgb {
KGB_GQ_LOOKUP_FIBRE_AND_RT
KGB_GQ_LOOKUP_ELEM
}  // namespace kgb
