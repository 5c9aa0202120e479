// Instantiations of the FP64 tensor-path forward kernels (dmma_kernels.cuh).
#include "dmma_kernels.cuh"

namespace kgb {

#define KGB_DMMA_CASES(NN)                                                 \
    case NN * 64 + 1 * 2: return fwd_dmma_kernel<NN, 1, false>;            \
    case NN * 64 + 2 * 2: return fwd_dmma_kernel<NN, 2, false>;            \
    case NN * 64 + 4 * 2: return fwd_dmma_kernel<NN, 4, false>;            \
    case NN * 64 + 8 * 2: return fwd_dmma_kernel<NN, 8, false>;
#define KGB_DMMA_CASES_FULL(NN)                                            \
    case NN * 64 + 1 * 2 + 1: return fwd_dmma_kernel<NN, 1, true>;         \
    case NN * 64 + 2 * 2 + 1: return fwd_dmma_kernel<NN, 2, true>;         \
    case NN * 64 + 4 * 2 + 1: return fwd_dmma_kernel<NN, 4, true>;         \
    case NN * 64 + 8 * 2 + 1: return fwd_dmma_kernel<NN, 8, true>;

DmmaFn fwd_dmma_lookup(int nn, int qt, bool full)
{
    switch (nn * 64 + qt * 2 + (full ? 1 : 0)) {
    KGB_DMMA_CASES(6)
    KGB_DMMA_CASES(7)
    KGB_DMMA_CASES_FULL(8)
    case 8 * 64 + 1 * 2: return fwd_dmma_kernel<8, 1, false>;  // d = 1
    KGB_DMMA_CASES_FULL(16)
    case 16 * 64 + 1 * 2: return fwd_dmma_kernel<16, 1, false>;  // d = 1
    default: return nullptr;
    }
}

DmmaFn fwd_dmma_global_lookup(int nn)
{
    switch (nn) {
    case 6: return fwd_dmma_global_kernel<6>;
    case 7: return fwd_dmma_global_kernel<7>;
    case 8: return fwd_dmma_global_kernel<8>;
    case 16: return fwd_dmma_global_kernel<16>;
    default: return nullptr;
    }
}

}  // namespace kgb
