// Grouped forward (and adjoint) plans: several groups of entries with different
// (d, n, fan-in) served by one run that can be captured in a CUDA graph.
//
// No reference counterpart: the reference serves one (d, n) per call with one CTA
// per entry (kronmult_gpu/kronmult.cu:173-197).  The plan gives every forward group a
// persistent kernel compiled for its n (grouped_kernels.cuh) with a device work
// queue; the run forks the groups' kernels (and any adjoint groups) into parallel
// branches and joins them back into the caller's stream.  Two output modes:
//  - atomic: runs of equal output pointers are summed in registers and added with
//    atomics (same semantics as kronmult_batched);
//  - deterministic: each group's entries are ordered by output pointer on the device
//    (a bitonic sort of (pointer, entry index) pairs, which equals a stable sort by
//    pointer) and every output vector is owned by one team, which sums its entries
//    in entry order (in shared memory) and adds the sum with one plain
//    read-modify-write: bitwise reproducible.
//    The forward groups then run one after another, so an output may also be
//    shared by groups.
#include <algorithm>
#include <climits>
#include <vector>
#include "df_common.cuh"
#include "fwd_launch.cuh"
#include "grouped.cuh"
#include "tuning.cuh"

namespace kgb {

// ---- device-side ordering by output pointer --------------------------------
namespace {

constexpr int kSortLocal = 2048;  // elements one CTA sorts in shared memory (1024 threads, 2 each)

__global__ void gq_sort_init(const void *const *out, long long nb, long long m, unsigned long long *keys,
                             long long *perm)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        keys[i] = i < nb ? (unsigned long long)reinterpret_cast<uintptr_t>(out[i]) : ~0ull;
        perm[i] = i;
    }
}

// (key, index) pairs in lexicographic order: equal keys keep their entry order
__device__ __forceinline__ bool pair_gt(unsigned long long ka, long long pa, unsigned long long kb, long long pb)
{
    return ka > kb || (ka == kb && pa > pb);
}

// one compare-exchange step of the bitonic network (partner distance j >= kSortLocal)
__global__ void gq_sort_step(unsigned long long *keys, long long *perm, long long m, long long j, long long k)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        const long long l = i ^ j;
        if (l <= i) continue;
        const unsigned long long ki = keys[i], kl = keys[l];
        const long long pi = perm[i], pl = perm[l];
        const bool up = (i & k) == 0;
        if (pair_gt(ki, pi, kl, pl) == up) {
            keys[i] = kl;
            keys[l] = ki;
            perm[i] = pl;
            perm[l] = pi;
        }
    }
}

// every step with partner distance j <= jmax (< kSortLocal) of the stages k in
// [k_first, k_last], inside one 2048-element chunk in shared memory
__global__ void __launch_bounds__(1024) gq_sort_local(unsigned long long *keys, long long *perm, long long k_first,
                                                      long long k_last, long long jmax)
{
    __shared__ unsigned long long sk[kSortLocal];
    __shared__ long long sp[kSortLocal];
    const long long base = (long long)blockIdx.x * kSortLocal;
    for (int t = threadIdx.x; t < kSortLocal; t += blockDim.x) {
        sk[t] = keys[base + t];
        sp[t] = perm[base + t];
    }
    __syncthreads();
    for (long long k = k_first; k <= k_last; k <<= 1) {
        for (long long j = (k >> 1) < jmax ? (k >> 1) : jmax; j > 0; j >>= 1) {
            const int t = threadIdx.x;  // pair t: positions i and i + j
            const int i = (int)((t / j) * 2 * j + (t % j));
            const int l = i + (int)j;
            const bool up = ((base + i) & k) == 0;
            const unsigned long long ki = sk[i], kl = sk[l];
            const long long pi = sp[i], pl = sp[l];
            if (pair_gt(ki, pi, kl, pl) == up) {
                sk[i] = kl;
                sk[l] = ki;
                sp[i] = pl;
                sp[l] = pi;
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < kSortLocal; t += blockDim.x) {
        keys[base + t] = sk[t];
        perm[base + t] = sp[t];
    }
}

// the group's pointer tables in sorted order
__global__ void gq_gather(const void *const *mats, const void *const *in, const void *const *out, int d, long long nb,
                          const long long *perm, const void **s_mats, const void **s_in, void **s_out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nb; k += (long long)gridDim.x * blockDim.x) {
        const long long p = perm[k];
        s_in[k] = in[p];
        s_out[k] = const_cast<void *>(out[p]);
        for (int i = 0; i < d; ++i) s_mats[k * d + i] = mats[p * d + i];
    }
}

}  // namespace

void gq_group_launch(const void *const *mats, const void *const *in, const void *const *out, int d, long long nb,
                     long long m, unsigned long long *keys, long long *perm, const void **s_mats,
                     const void **s_in, void **s_out, cudaStream_t st)
{
    const unsigned grid = (unsigned)std::min<long long>((m + 255) / 256, 4096);
    gq_sort_init<<<grid, 256, 0, st>>>(out, nb, m, keys, perm);
    const unsigned chunks = (unsigned)(m / kSortLocal);
    // stages up to kSortLocal entirely inside the chunks
    gq_sort_local<<<chunks, 1024, 0, st>>>(keys, perm, 2, kSortLocal, kSortLocal / 2);
    for (long long k = 2 * kSortLocal; k <= m; k <<= 1) {
        for (long long j = k >> 1; j >= kSortLocal; j >>= 1) gq_sort_step<<<grid, 256, 0, st>>>(keys, perm, m, j, k);
        gq_sort_local<<<chunks, 1024, 0, st>>>(keys, perm, k, k, kSortLocal / 2);
    }
    const unsigned ggrid = (unsigned)std::min<long long>((nb + 255) / 256, 4096);
    gq_gather<<<ggrid, 256, 0, st>>>(mats, in, out, d, nb, perm, s_mats, s_in, s_out);
}

// ---- deterministic mode, second pass ----------------------------------------
namespace {

// Thread (u, i): when the segment ending unit u continues into unit u+1 and started in
// unit u, add element i of its partials -- slot 2u+1, then slot 2v of every following
// unit v it covers, in order -- into the output with one plain read-modify-write.
template <typename T, typename TO> __global__ void gq_seg_reduce(const GqArgs a)
{
    const unsigned long long *k = a.keys;
    const T *part = reinterpret_cast<const T *>(a.partial);
    const long long total = a.n_units * (long long)a.N;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long u = idx / a.N;
        const int i = (int)(idx - u * a.N);
        const long long b = u * a.unit, e = b + a.unit < a.nb ? b + a.unit : a.nb;
        if (e >= a.nb || k[e - 1] != k[e]) continue;                    // does not continue into u+1
        if (b > 0 && k[b - 1] == k[b] && k[b] == k[e - 1]) continue;    // started before unit u
        T s = part[(2 * u + 1) * a.N + i];
        for (long long v = u + 1;; ++v) {
            const long long vb = v * a.unit, ve = vb + a.unit < a.nb ? vb + a.unit : a.nb;
            s += part[(2 * v) * a.N + i];
            if (!(ve < a.nb && k[vb] == k[ve - 1] && k[ve - 1] == k[ve])) break;  // ends in unit v
        }
        TO *o = reinterpret_cast<TO *>(static_cast<uintptr_t>(k[e - 1]));
        o[i] = o[i] + (TO)s;
    }
}

}  // namespace

void gq_seg_reduce_launch(const GqArgs &a, int dtype, cudaStream_t st)
{
    const long long total = a.n_units * (long long)a.N;
    const unsigned grid = (unsigned)std::min<long long>((total + 255) / 256, 8192);
    if (dtype == KRONMULT_DTYPE_F64 || dtype == KRONMULT_DTYPE_F64_EMULATED)
        gq_seg_reduce<double, double><<<grid, 256, 0, st>>>(a);
    else
        gq_seg_reduce<float, float><<<grid, 256, 0, st>>>(a);
}

// ---- planning ----------------------------------------------------------------

namespace {

struct GqShape {
    GqFn fn = nullptr;
    int ts = 0, team_elems = 0, vec_pad = 0;
    int block = kGroupedBlock;  // threads per CTA: a multiple of ts
};

// The single-call planner's choice, for one team per entry at a time: fibre mapping
// with a compile-time n (team size from the same target of fibres per thread), or
// for FP64 the element mapping when it uses the lanes clearly better (by > 5
// points); n = 9..16 take the element mapping with n at run time.
template <typename T, typename TO>
int gq_shape(int d, int n, bool det, const kronmult_tuning *tune, GqShape &sh)
{
    const long long Nl = pow_ll(n, d);
    if (n < 2 || n > 16 || d < 1 || Nl > (long long)INT_MAX) return cudaErrorNotSupported;
    const int N = (int)Nl, F = N / n;
    const bool forced = tune && tune->team_size > 0;
    constexpr int kAlign = 16 / (int)sizeof(T);
    sh.vec_pad = round_up(N, kAlign);
    // [vector | factors], and in the deterministic mode (n <= 8) a run accumulator of
    // vec_pad values at the end of the slice
    sh.team_elems = sh.vec_pad + round_up(d * n * n, kAlign) + (det && n <= 8 ? sh.vec_pad : 0);
    if (n > 8) {
        const int ts = elem_team_size(N, 16, forced ? tune->team_size : 0, kGroupedBlock);
        if (ts == 0) return cudaErrorNotSupported;
        const int per = (N + ts - 1) / ts;
        int emax = 1;
        while (emax < per) emax *= 2;
        sh.fn = gq_elem_rt_lookup<T, TO>(emax, det);
        sh.ts = ts;
        return sh.fn ? cudaSuccess : cudaErrorNotSupported;
    }
    const int qcap = (n <= 4) ? 8 : 4;
    int ts = 8;
    if (forced) {
        ts = tune->team_size;
        while (ts < kGroupedBlock && (F + ts - 1) / ts > qcap) ts *= 2;
    } else {
        const int qtarget = (n <= 4 || (n == 6 && sizeof(T) == 8)) ? 4 : 2;
        while (ts < kGroupedBlock && (long long)ts * qtarget < F) ts *= 2;
    }
    if (ts > kGroupedBlock) return cudaErrorNotSupported;
    const int q = (F + ts - 1) / ts;
    int qmax = 1;
    while (qmax < q) qmax *= 2;
    if (qmax > qcap) return cudaErrorNotSupported;
    sh.fn = gq_fibre_lookup<T, TO>(n, qmax, det);
    sh.ts = ts;
    const int fmap = fp64_mapping(tune);
    if (sizeof(T) == 8 && fmap != 3 && (fmap == 4 || !forced)) {
        const double fibre_util = lane_use(F, ts);
        int tse = 8;
        if (fmap == 4 && forced) {
            tse = tune->team_size;
            while (tse < kGroupedBlock && (N + tse - 1) / tse > 8) tse *= 2;
        } else {
            while (tse < kGroupedBlock && (N + tse - 1) / tse > 4) tse *= 2;
        }
        const int per = (N + tse - 1) / tse;
        const double util_e = lane_use(N, tse);
        // ties go to the element mapping here: on C3's groups (d, n) = (2,8), (4,4) its
        // persistent kernels measured 3-9 % faster at equal lane use
        if (tse <= kGroupedBlock && per <= 8 && (fmap == 4 || util_e >= fibre_util)) {
            int emax = 1;
            while (emax < per) emax *= 2;
            const GqFn fe = gq_elem_lookup<T, TO>(n, emax, det);
            if (fe) {
                sh.fn = fe;
                sh.ts = tse;
                sh.team_elems += sh.vec_pad;  // the element kernels ping-pong between two vectors
                // The rows form: the smallest power-of-two team of whole warps that is a
                // multiple of n and leaves at most 4 elements per thread, at the same lane
                // use (issued warp rounds); each thread then keeps its factor row in
                // registers.  (n = 2, 4, 8; d=2 n=8 measured 2 % faster.  Teams of 96 or
                // 192 threads for n = 3, 6 measured 1-6 % slower: fewer warps per SM.)
                if (!(forced && fmap == 4)) {
                    for (int tr = 32; tr <= kGroupedBlock; tr *= 2) {
                        const int pr = (N + tr - 1) / tr;
                        if (tr % n != 0 || pr > 4 || lane_use(N, tr) < lane_use(N, tse) - 1e-9) continue;
                        int er = 2;
                        while (er < pr) er *= 2;
                        const GqFn fr = gq_elem_rows_lookup<T, TO>(n, er, det);
                        if (fr) {
                            sh.fn = fr;
                            sh.ts = tr;
                            sh.block = kGroupedBlock / tr * tr;
                        }
                        break;
                    }
                }
            }
        }
    }
    return sh.fn ? cudaSuccess : cudaErrorNotSupported;
}

// Double-float shape: the single-call emulated path's team (whole fibres, at most 4
// per thread), the slice df_entry wants plus, in deterministic mode, N FP64 run sums.
int gq_df_shape(int d, int n, bool det, const kronmult_tuning *tune, GqShape &sh)
{
    const long long Nl = pow_ll(n, d);
    if (n < 2 || n > 8 || d < 1 || Nl > (long long)INT_MAX) return cudaErrorNotSupported;
    const int N = (int)Nl, F = N / n;
    int qmax = 0;
    int ts = df_team(F, qmax);
    if (tune && tune->team_size > 0 && ts) {
        ts = std::max(ts, std::min(tune->team_size, kGroupedBlock));
        const int q = (F + ts - 1) / ts;
        qmax = 1;
        while (qmax < q) qmax *= 2;
    }
    if (!ts || ts > kGroupedBlock) return cudaErrorNotSupported;
    sh.vec_pad = round_up(N, 4);
    sh.team_elems = df_slice_floats(d, n, sh.vec_pad) + (det ? 2 * round_up(N, 2) : 0);
    sh.fn = gq_df_lookup(n, qmax, det);
    sh.ts = ts;
    return sh.fn ? cudaSuccess : cudaErrorNotSupported;
}

int shape_for(int dtype, int d, int n, bool det, const kronmult_tuning *tune, GqShape &sh)
{
    if (dtype == KRONMULT_DTYPE_F64_EMULATED) return gq_df_shape(d, n, det, tune, sh);
    return dtype == KRONMULT_DTYPE_F64 ? gq_shape<double, double>(d, n, det, tune, sh)
                                       : gq_shape<float, float>(d, n, det, tune, sh);
}

long long pow2_ceil(long long v)
{
    long long p = 1;
    while (p < v) p <<= 1;
    return p;
}

void destroy_plan(GroupedPlan *pl)
{
    if (!pl) return;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != pl->device) cudaSetDevice(pl->device);
    for (cudaStream_t s : pl->branches)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : pl->joins)
        if (e) cudaEventDestroy(e);
    if (pl->fork) cudaEventDestroy(pl->fork);
    if (pl->dmem) cudaFree(pl->dmem);
    if (dev != pl->device) cudaSetDevice(dev);
    delete pl;
}

int run_adjoint(int dtype, const kronmult_adjoint_group &g, cudaStream_t st)
{
    if (dtype != KRONMULT_DTYPE_F32)  // FP64 data (native or emulated forward): the FP64 adjoint
        return kronmult_batched_adjoint_f64_async(
            g.matrix_count, g.matrix_size, reinterpret_cast<const double *const *>(g.matrix_list_batched),
            g.matrix_stride, reinterpret_cast<const double *const *>(g.input_batched),
            reinterpret_cast<const double *const *>(g.grad_output_batched),
            reinterpret_cast<double *const *>(g.grad_input_batched),
            reinterpret_cast<double *const *>(g.grad_matrix_list_batched), g.grad_matrix_stride, g.nb_batch, st,
            nullptr);
    return kronmult_batched_adjoint_f32_async(
        g.matrix_count, g.matrix_size, reinterpret_cast<const float *const *>(g.matrix_list_batched),
        g.matrix_stride, reinterpret_cast<const float *const *>(g.input_batched),
        reinterpret_cast<const float *const *>(g.grad_output_batched),
        reinterpret_cast<float *const *>(g.grad_input_batched),
        reinterpret_cast<float *const *>(g.grad_matrix_list_batched), g.grad_matrix_stride, g.nb_batch, st, nullptr);
}

}  // namespace

int grouped_plan_create(GroupedPlan *&out, const kronmult_group *groups, int n_groups,
                        const kronmult_adjoint_group *adj, int n_adj, int dtype, int mode,
                        const kronmult_tuning *tunings)
{
    out = nullptr;
    if (n_groups < 0 || (n_groups > 0 && !groups) || n_adj < 0 || (n_adj > 0 && !adj)) return cudaErrorInvalidValue;
    if (dtype != KRONMULT_DTYPE_F64 && dtype != KRONMULT_DTYPE_F32 && dtype != KRONMULT_DTYPE_F64_EMULATED)
        return cudaErrorInvalidValue;
    if (mode != KRONMULT_MODE_ATOMIC && mode != KRONMULT_MODE_DETERMINISTIC) return cudaErrorInvalidValue;
    const bool det = mode == KRONMULT_MODE_DETERMINISTIC;
    // bytes of a shared-memory element (floats for the double-float kernels) and of a
    // run sum / partial-slot value (FP64 for both FP64 forms)
    const int elem = dtype == KRONMULT_DTYPE_F64 ? 8 : 4;
    const int acc_elem = dtype == KRONMULT_DTYPE_F32 ? 4 : 8;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);

    auto *pl = new GroupedPlan();
    pl->dtype = dtype;
    pl->mode = mode;
    pl->device = dev;
    int rc = cudaSuccess;
    for (int g = 0; g < n_groups && rc == cudaSuccess; ++g) {
        const kronmult_group &G = groups[g];
        if (G.matrix_count < 0 || G.matrix_size < 0 || G.nb_batch < 0 ||
            G.matrix_stride < (G.matrix_size > 0 ? G.matrix_size : 1)) {
            rc = cudaErrorInvalidValue;
            break;
        }
        if (G.nb_batch == 0 || G.matrix_size == 0) continue;  // nothing to add
        if (!G.matrix_list_batched || !G.input_batched || !G.output_batched) {
            rc = cudaErrorInvalidValue;
            break;
        }
        kronmult_tuning tt{};
        const kronmult_tuning *tp =
            (tunings && (tunings[g].team_size > 0 || fp64_mapping(&tunings[g]))) ? &tunings[g] : nullptr;
        if (!tp && tuning_cache_lookup(G.matrix_count, G.matrix_size, dtype, tt) && tt.team_size <= kGroupedBlock)
            tp = &tt;
        GqShape sh;
        rc = shape_for(dtype, G.matrix_count, G.matrix_size, det, tp, sh);
        if (rc != cudaSuccess) break;
        const int teams = sh.block / sh.ts;
        const size_t smem = (size_t)teams * sh.team_elems * elem;
        if (smem > (size_t)di.max_smem_optin || !ensure_smem_attr((const void *)sh.fn, smem)) {
            rc = cudaErrorNotSupported;
            break;
        }
        GqLaunch L;
        L.fn = sh.fn;
        L.smem = smem;
        L.block = sh.block;
        int per_sm = std::max(1, occupancy((const void *)sh.fn, sh.block, smem));
        if (tunings && tunings[g].ctas_per_sm > 0) per_sm = std::min(per_sm, tunings[g].ctas_per_sm);
        L.grid = di.sms * per_sm;
        GqArgs &a = L.args;
        a.mats = G.matrix_list_batched;
        a.in = G.input_batched;
        a.out = G.output_batched;
        a.nb = G.nb_batch;
        a.d = G.matrix_count;
        a.n = G.matrix_size;
        a.stride = G.matrix_stride;
        a.N = (int)pow_ll(G.matrix_size, G.matrix_count);
        a.team_size = sh.ts;
        a.team_elems = sh.team_elems;
        a.vec_pad = sh.vec_pad;
        // Unit size, unless tuned: FP64 atomic mode takes one entry per unit (the queue
        // then evens out the tail to one entry; measured 2-6 % faster than four units per
        // team on C3's groups, where an entry is 1-15 us of FP64 work); otherwise about
        // four units per resident team (deterministic mode sums runs within a unit, and
        // single entries measured up to 14 % slower there).
        const long long teams_total = (long long)L.grid * teams;
        long long unit = (a.nb + 4 * teams_total - 1) / (4 * teams_total);
        if (dtype != KRONMULT_DTYPE_F32 && !det) unit = 1;
        if (tunings && tunings[g].entries_per_team > 0) unit = tunings[g].entries_per_team;
        a.unit = std::max(1LL, unit);
        a.n_units = (a.nb + a.unit - 1) / a.unit;
        if (a.n_units > (long long)UINT_MAX - (1LL << 24)) {  // room for every team's claim ahead
            rc = cudaErrorInvalidValue;
            break;
        }
        if (det) {
            L.sort_m = std::max<long long>(kSortLocal, pow2_ceil(a.nb));
            a.snap = G.matrix_size > 8 ? 1 : 0;  // run-time n: whole segments per unit
        }
        pl->launches.push_back(L);
        pl->n_units += a.n_units;
        pl->grid_max = std::max(pl->grid_max, L.grid);
        pl->smem_max = std::max(pl->smem_max, smem);
    }
    for (int g = 0; g < n_adj && rc == cudaSuccess; ++g) {
        const kronmult_adjoint_group &A = adj[g];
        if (A.matrix_count < 0 || A.matrix_size < 0 || A.nb_batch < 0 ||
            A.matrix_stride < (A.matrix_size > 0 ? A.matrix_size : 1))
            rc = cudaErrorInvalidValue;
        else if (A.nb_batch > 0)
            pl->adjoints.push_back(GqAdjoint{A});
    }
    if (rc != cudaSuccess) {
        destroy_plan(pl);
        return rc;
    }

    // device memory: the queue counters, then each deterministic group's sort buffers
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t total = align(std::max<size_t>(1, pl->launches.size()) * sizeof(unsigned));
    for (const GqLaunch &L : pl->launches)
        if (L.sort_m)
            total += align((size_t)L.sort_m * 8) * 2 + align((size_t)L.args.nb * (L.args.d + 2) * 8) +
                     (L.args.snap ? 0 : align((size_t)2 * L.args.n_units * L.args.N * acc_elem));
    if (cudaMalloc(&pl->dmem, total) != cudaSuccess) {
        cudaGetLastError();
        destroy_plan(pl);
        return cudaErrorMemoryAllocation;
    }
    char *p = static_cast<char *>(pl->dmem);
    pl->counters = reinterpret_cast<unsigned *>(p);
    p += align(std::max<size_t>(1, pl->launches.size()) * sizeof(unsigned));
    for (size_t i = 0; i < pl->launches.size(); ++i) {
        GqLaunch &L = pl->launches[i];
        L.args.queue = pl->counters + i;
        if (L.sort_m) {
            L.keys = reinterpret_cast<unsigned long long *>(p);
            p += align((size_t)L.sort_m * 8);
            L.perm = reinterpret_cast<long long *>(p);
            p += align((size_t)L.sort_m * 8);
            const long long nb = L.args.nb;
            L.s_mats = reinterpret_cast<const void **>(p);
            L.s_in = L.s_mats + nb * L.args.d;
            L.s_out = const_cast<void **>(L.s_in + nb);
            p += align((size_t)nb * (L.args.d + 2) * 8);
            if (!L.args.snap) {
                L.args.partial = p;
                p += align((size_t)2 * L.args.n_units * L.args.N * acc_elem);
            }
            L.mats = L.args.mats;
            L.in = L.args.in;
            L.out = L.args.out;
            L.args.mats = L.s_mats;
            L.args.in = L.s_in;
            L.args.out = L.s_out;
            L.args.keys = L.keys;
            pl->n_sorted += nb;
        }
    }
    // one branch stream and join event per parallel kernel, one fork event
    const size_t n_branches = (det ? 0 : pl->launches.size()) + pl->adjoints.size();
    pl->branches.assign(std::max<size_t>(1, n_branches), nullptr);
    pl->joins.assign(pl->branches.size(), nullptr);
    cudaError_t e = cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming);
    for (size_t i = 0; i < pl->branches.size() && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&pl->branches[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->joins[i], cudaEventDisableTiming);
    }
    // deterministic mode: order the entries on the device and wait (no copy to the host)
    if (e == cudaSuccess && det) {
        for (const GqLaunch &L : pl->launches)
            gq_group_launch(L.mats, L.in, L.out, L.args.d, L.args.nb, L.sort_m, L.keys, L.perm, L.s_mats, L.s_in,
                            L.s_out, pl->branches[0]);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(pl->branches[0]);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        destroy_plan(pl);
        return e;
    }
    out = pl;
    return cudaSuccess;
}

int grouped_regroup(const GroupedPlan *pl, cudaStream_t st)
{
    if (!pl) return cudaErrorInvalidValue;
    for (const GqLaunch &L : pl->launches)
        if (L.sort_m)
            gq_group_launch(L.mats, L.in, L.out, L.args.d, L.args.nb, L.sort_m, L.keys, L.perm, L.s_mats, L.s_in,
                            L.s_out, st);
    return (int)cudaGetLastError();
}

int grouped_run(const GroupedPlan *pl, cudaStream_t st)
{
    if (!pl) return cudaErrorInvalidValue;
    const bool det = pl->mode == KRONMULT_MODE_DETERMINISTIC;
    cudaError_t e = cudaSuccess;
    if (!pl->launches.empty()) e = cudaMemsetAsync(pl->counters, 0, pl->launches.size() * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    auto launch = [&](const GqLaunch &L, cudaStream_t s) {
        L.fn<<<L.grid, L.block, L.smem, s>>>(L.args);
        return cudaGetLastError();
    };
    const size_t n_par = (det ? 0 : pl->launches.size()) + pl->adjoints.size();
    if (n_par > 0 && (e = cudaEventRecord(pl->fork, st)) != cudaSuccess) return e;
    size_t b = 0;
    auto branch = [&](auto &&enqueue) -> cudaError_t {
        cudaStream_t s = pl->branches[b];
        cudaError_t r = cudaStreamWaitEvent(s, pl->fork, 0);
        if (r == cudaSuccess) r = (cudaError_t)enqueue(s);
        if (r == cudaSuccess) r = cudaEventRecord(pl->joins[b], s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(st, pl->joins[b], 0);
        ++b;
        return r;
    };
    for (const GqLaunch &L : pl->launches) {
        if (det) {
            e = launch(L, st);
            if (e == cudaSuccess && L.args.partial) {
                gq_seg_reduce_launch(L.args, pl->dtype, st);
                e = cudaGetLastError();
            }
        } else {
            e = branch([&](cudaStream_t s) { return (int)launch(L, s); });
        }
        if (e != cudaSuccess) return e;
    }
    for (const GqAdjoint &A : pl->adjoints) {
        e = branch([&](cudaStream_t s) { return run_adjoint(pl->dtype, A.g, s); });
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kronmult_grouped_plan_create(kronmult_grouped_plan *plan, const kronmult_group *groups, int n_groups, int dtype,
                                 int mode, const kronmult_tuning *tunings)
{
    return kronmult_grouped_plan_create_with_adjoint(plan, groups, n_groups, nullptr, 0, dtype, mode, tunings);
}

int kronmult_grouped_plan_create_with_adjoint(kronmult_grouped_plan *plan, const kronmult_group *groups,
                                              int n_groups, const kronmult_adjoint_group *adjoint_groups,
                                              int n_adjoint, int dtype, int mode, const kronmult_tuning *tunings)
{
    if (!plan) return cudaErrorInvalidValue;
    GroupedPlan *pl = nullptr;
    const int rc = grouped_plan_create(pl, groups, n_groups, adjoint_groups, n_adjoint, dtype, mode, tunings);
    *plan = reinterpret_cast<kronmult_grouped_plan>(pl);
    return rc;
}

int kronmult_grouped_run(kronmult_grouped_plan plan, void *stream)
{
    return grouped_run(reinterpret_cast<const GroupedPlan *>(plan), (cudaStream_t)stream);
}

int kronmult_grouped_regroup(kronmult_grouped_plan plan, void *stream)
{
    return grouped_regroup(reinterpret_cast<const GroupedPlan *>(plan), (cudaStream_t)stream);
}

int kronmult_grouped_plan_info(kronmult_grouped_plan plan, long long *info, int n_info)
{
    auto *pl = reinterpret_cast<const GroupedPlan *>(plan);
    if (!pl || !info) return cudaErrorInvalidValue;
    int block_max = 0;
    for (const GqLaunch &L : pl->launches) block_max = std::max(block_max, L.block);
    const long long v[6] = {pl->grid_max, block_max ? block_max : kGroupedBlock, (long long)pl->smem_max,
                            pl->n_units, (long long)(pl->launches.size() + pl->adjoints.size()), pl->n_sorted};
    for (int i = 0; i < n_info && i < 6; ++i) info[i] = v[i];
    return cudaSuccess;
}

int kronmult_grouped_plan_destroy(kronmult_grouped_plan plan)
{
    destroy_plan(reinterpret_cast<GroupedPlan *>(plan));
    return cudaSuccess;
}

}  // extern "C"
