// Allocation-free forward: kronmult_batched_f64_noalloc.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they run
// the product -- code that runs inside a memory pool or arena owned by the
// application (ASGarD-style solvers that size all device memory up front),
// callbacks that must not touch the allocator, and runtimes that forbid device
// allocation after start-up.  The grouped forward needs device scratch for its
// work list, which its plan allocates; this variant keeps that scratch in a
// fixed array compiled into the library instead, so a call allocates nothing.
//
// What it computes: the same as kronmult_batched_f64 (output[k] += kron(A_k).input[k],
// atomic into shared outputs).  Work is scheduled by output run, as in the
// deterministic grouped mode: a first kernel lists the start of every piece of work,
// a persistent kernel hands the pieces to teams through a queue counter, and each
// team sums its piece in entry order and adds the sum with one atomic per element.
// A piece is a run of consecutive entries with the same output pointer, cut where
// the entry index is a multiple of kNaPiece (16) and the run already holds more than
// 16 entries, so that one long run (the reference's benchmarks send thousands of
// entries into 5 outputs) is spread over many teams instead of serialising on one.
// When every output's entries are one contiguous run of at most 16 entries, each
// output element receives exactly one addition and the result is bitwise
// reproducible.
//
// Scratch: g_noalloc_scratch below, 4 MiB + 256 bytes, holding two counters and
// up to KRONMULT_NOALLOC_MAX_ENTRIES run starts.  Every GPU that loads the library
// holds this array until the process exits.  All calls share it and it keeps the
// last call's contents; the counters are cleared at the start of every call.
// Calls that overlap on the GPU (concurrent streams, or several host threads)
// race on the array and must be serialised by the caller.
#include <climits>
#include "fwd_kernels.cuh"
#include "kronmult_gb300.h"

// [0, 256): counters (run count, queue head); [256, ...): run start indices
static __device__ __align__(256) unsigned char g_noalloc_scratch[256 + (size_t)KRONMULT_NOALLOC_MAX_ENTRIES * sizeof(int)];

namespace kgb {
namespace {

constexpr int kNaBlock = 256;
constexpr int kNaPiece = 16;  // longest piece of a long run that one team sums before its atomics

// Entry k starts a piece: it is the first entry, its output differs from entry k-1's, or
// k is a multiple of kNaPiece and entry k-kNaPiece adds into the same output (so the run
// around k is longer than kNaPiece).  Runs of at most kNaPiece entries are never cut.
__device__ __forceinline__ bool piece_start(double *const *out, int k)
{
    if (k == 0) return true;
    const double *o = out[k];
    if (out[k - 1] != o) return true;
    return (k % kNaPiece) == 0 && out[k - kNaPiece] == o;
}

struct NaArgs {
    const double *const *mats;
    const double *const *in;
    double *const *out;
    unsigned *counters;
    int *runs;
    int nb, d, stride, N, team_size, team_elems, vec_pad;
};

// piece starts, in no particular order
__global__ void noalloc_runs_kernel(const NaArgs a)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nb; k += gridDim.x * blockDim.x) {
        if (piece_start(a.out, k)) {
            const unsigned slot = atomicAdd(&a.counters[0], 1u);
            a.runs[slot] = k;
        }
    }
}

template <int NN, int QMAX> __global__ void __launch_bounds__(kNaBlock) noalloc_fwd_kernel(const NaArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_run[kNaBlock / 8];
    const Team tm(a.team_size);
    double *buf = reinterpret_cast<double *>(smem_raw) + (size_t)tm.id * a.team_elems;
    const unsigned n_runs = a.counters[0];
    for (;;) {
        if (tm.rank == 0) {
            const unsigned q = atomicAdd(&a.counters[1], 1u);
            s_run[tm.id] = q < n_runs ? a.runs[q] : -1;
        }
        tm.sync();
        const int start = s_run[tm.id];
        tm.sync();
        if (start < 0) break;
        int end = start + 1;
        while (end < a.nb && !piece_start(a.out, end)) ++end;
        team_forward<double, double, NN, QMAX, false>(a.mats, a.in, a.out, nullptr, a.d, a.stride, a.N, start, end,
                                                      buf, buf + a.vec_pad, tm);
    }
}

using NaFn = void (*)(const NaArgs);

NaFn noalloc_lookup(int nn, int qmax)
{
#define KGB_NA(NN, Q) \
    case NN * 16 + Q: return noalloc_fwd_kernel<NN, Q>;
    switch (nn * 16 + qmax) {
        KGB_NA(2, 1) KGB_NA(2, 2) KGB_NA(2, 4)
        KGB_NA(3, 1) KGB_NA(3, 2) KGB_NA(3, 4)
        KGB_NA(4, 1) KGB_NA(4, 2) KGB_NA(4, 4)
        KGB_NA(5, 1) KGB_NA(5, 2) KGB_NA(5, 4)
        KGB_NA(6, 1) KGB_NA(6, 2) KGB_NA(6, 4)
        KGB_NA(7, 1) KGB_NA(7, 2) KGB_NA(7, 4)
        KGB_NA(8, 1) KGB_NA(8, 2) KGB_NA(8, 4)
    default: return nullptr;
    }
#undef KGB_NA
}

// Device address of the scratch array in the current device's context, looked up on
// every call (host code cannot use the array's name as a device address).  The lookup
// allocates nothing and keeps no state, so concurrent calls from several host threads
// need no lock and a context re-created after cudaDeviceReset is never served a stale
// address.
int scratch_address(void **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();  // leave no sticky status behind for later, unrelated calls
        return e;
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" int kronmult_batched_f64_noalloc(int matrix_count, int matrix_size,
                                            const double *const *matrix_list_batched, int matrix_stride,
                                            const double *const *input_batched, double *const *output_batched,
                                            int nb_batch, void *stream)
{
    const int d = matrix_count, n = matrix_size;
    if (d < 0 || n < 0 || nb_batch < 0 || matrix_stride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    if (nb_batch > KRONMULT_NOALLOC_MAX_ENTRIES) return cudaErrorInvalidValue;  // beyond the scratch array
    long long Nl = 1;
    for (int i = 0; i < d && Nl <= INT_MAX; ++i) Nl *= n;
    if (Nl > INT_MAX) return cudaErrorInvalidValue;
    if (nb_batch == 0 || n == 0) return cudaSuccess;
    if (!matrix_list_batched || !input_batched || !output_batched) return cudaErrorInvalidValue;
    if (n < 2 || n > 8 || d < 1) return cudaErrorNotSupported;
    const int N = (int)Nl, F = N / n;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    void *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != cudaSuccess) return rc;
    int sms = 0, smem_optin = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);

    // team shape: the forward's heuristic, at most 4 fibres per thread
    const int qtarget = (n <= 4) ? 4 : 2;
    int ts = 8;
    while (ts < kNaBlock && ts * qtarget < F) ts *= 2;
    while (ts < kNaBlock && (F + ts - 1) / ts > 4) ts *= 2;
    const int q = (F + ts - 1) / ts;
    int qmax = 1;
    while (qmax < q) qmax *= 2;
    if (qmax > 4) return cudaErrorNotSupported;
    const int vpad = (N + 1) & ~1;
    const int team_elems = vpad + ((d * n * n + 1) & ~1);
    int teams = kNaBlock / ts;
    while (teams > 1 && (size_t)teams * team_elems * sizeof(double) + 256 > (size_t)smem_optin) teams /= 2;
    const size_t smem = (size_t)teams * team_elems * sizeof(double);
    if (smem + 256 > (size_t)smem_optin) return cudaErrorNotSupported;  // 256 B kept for the static run slots
    const NaFn fn = noalloc_lookup(n, qmax);
    if (!fn) return cudaErrorNotSupported;
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) {
        cudaGetLastError();  // clear it: the status is returned here, not left for a later call
        return e;
    }
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, teams * ts, smem)) != cudaSuccess) {
        cudaGetLastError();
        return e;
    }
    if (per_sm < 1) per_sm = 1;

    NaArgs a{};
    a.mats = matrix_list_batched;
    a.in = input_batched;
    a.out = output_batched;
    a.counters = static_cast<unsigned *>(scratch);
    a.runs = reinterpret_cast<int *>(static_cast<unsigned char *>(scratch) + 256);
    a.nb = nb_batch;
    a.d = d;
    a.stride = matrix_stride;
    a.N = N;
    a.team_size = ts;
    a.team_elems = team_elems;
    a.vec_pad = vpad;

    cudaStream_t st = (cudaStream_t)stream;
    if ((e = cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) {
        cudaGetLastError();
        return e;
    }
    const int grid_runs = (nb_batch + 255) / 256 < sms * 4 ? (nb_batch + 255) / 256 : sms * 4;
    noalloc_runs_kernel<<<grid_runs, 256, 0, st>>>(a);
    fn<<<sms * per_sm, teams * ts, smem, st>>>(a);
    return (int)cudaGetLastError();
}
