// Explicit instantiation of the adjoint kernels for double.
#include "adj_kernels.cuh"
KGB_ADJ_INSTANTIATE_NN(double)

namespace kgb {
// the FP64 adjoint always uses the element-mapped kernel
template <> AdjFn<double> adj_fibre_lookup<double>(int, int) { return nullptr; }
}  // namespace kgb
