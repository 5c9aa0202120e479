// Per-group persistent kernels of the grouped forward (no reference counterpart;
// the reference serves one (d, n) per call, kronmult_gpu/kronmult.cu:173-197).
//
// Every group gets a kernel compiled for its own factor size n, with its own
// register budget, instead of one kernel that takes n at run time: the planner
// launches one such kernel per group, as parallel branches of one graph (atomic
// mode) or one after another (deterministic mode).  Each kernel is persistent: a
// team takes the next work unit from the group's device queue (one atomicAdd by
// the team's first thread), computes it with the same team forward as the
// single-call path (entries staged in shared memory, the d modes in place) and takes
// the next, until the queue is empty.
#pragma once
#include "grouped.cuh"

namespace kgb {

// A team's claims on the queue run one unit ahead: rank 0 claims the next unit while the
// team computes the current one, so the atomic's round trip to L2 overlaps work instead
// of stalling the team once per unit (units are single entries in the FP64 atomic mode).
// A team holding a claim beyond the queue's end stops; the counter may pass n_units by
// at most one claim per team (it is reset before every run).
__device__ __forceinline__ unsigned gq_first_claim(const GqArgs &a, const Team &tm)
{
    return tm.rank == 0 ? atomicAdd(a.queue, 1u) : 0u;
}

// the team's next unit as [b, e) of the group's order; false when the queue is empty
__device__ __forceinline__ bool gq_next(const GqArgs &a, long long *slot, const Team &tm, unsigned &claim,
                                        long long &b, long long &e)
{
    if (tm.rank == 0) {
        *slot = (long long)claim;
        if ((long long)claim < a.n_units) claim = atomicAdd(a.queue, 1u);  // the unit after this one
    }
    tm.sync();
    const long long u = *slot;
    tm.sync();
    if (u >= a.n_units) return false;
    b = u * a.unit;
    e = b + a.unit < a.nb ? b + a.unit : a.nb;
    if (a.snap) {  // first positions >= b and >= e that start a segment: whole segments per unit
        while (b > 0 && b < a.nb && a.keys[b] == a.keys[b - 1]) ++b;
        while (e > 0 && e < a.nb && a.keys[e] == a.keys[e - 1]) ++e;
    }
    return true;
}

// Adds one entry's result element y (at position p) into the output.  Atomic mode:
// with an atomic addition.  Deterministic mode, where the team owns this run and
// takes its entries in entry order: into the run sum `acc` in shared memory (each
// thread always owns the same elements, so no barrier is needed); at the run's last
// entry the sum goes into the output with one plain read-modify-write, or into the
// partial slot `part` when the run crosses a unit boundary.
template <typename T, typename TO, bool DET>
__device__ __forceinline__ void gq_add(TO *o, T *acc, T *part, int p, T y, bool first, bool last)
{
    if constexpr (DET) {
        const T s = first ? y : acc[p] + y;
        if (!last)
            acc[p] = s;
        else if (part)
            part[p] = s;
        else
            o[p] = o[p] + (TO)s;
    } else {
        atomic_add<TO>(o + p, (TO)y);
    }
}

// One entry, fibre mapping: the body of fwd_single_kernel.
template <typename T, typename TO, int NN, int QMAX, bool DET>
__device__ __forceinline__ void gq_entry_fibre(const T *const *mats, const T *const *in, TO *const *out, int d,
                                               int stride, int N, long long e, T *buf, T *fac, T *acc, T *part,
                                               bool first, bool last, const Team &tm)
{
    const int F = N / NN;
    constexpr bool kSwz = VecSwizzle<T, NN>::on;
    stage_vector<T, kSwz>(buf, in[e], N, tm);
    stage_factors<T, NN>(fac, mats + e * d, d, stride, tm);
    tm.sync();
    T y[QMAX][NN];
    for (int i = d - 1; i >= 0; --i) {
        const T *M = fac + i * NN * NN;
        mode_team<T, NN, QMAX, kSwz, !FactorInSmem<T, NN>::value>(buf, M, M, F, tm, y);
        tm.sync();  // every read of buf (and fac) for this mode is done
        if (i > 0) {
#pragma unroll
            for (int q = 0; q < QMAX; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
#pragma unroll
                    for (int r = 0; r < NN; ++r) buf[vec_pos<T, kSwz>(c + r * F)] = y[q][r];
                }
            }
            tm.sync();
        }
    }
    TO *o = out[e];
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
#pragma unroll
            for (int r = 0; r < NN; ++r) gq_add<T, TO, DET>(o, acc, part, c + r * F, y[q][r], first, last);
        }
    }
}

// One entry, element mapping with compile-time n (the arithmetic of
// fwd_single_elem_kernel), ping-ponging between two vector buffers: each output element
// goes to the other buffer as soon as it is computed (the last mode's straight into the
// output), so a mode ends with one barrier and no results wait in registers.  The
// barrier before staging keeps the previous entry's last reads ahead of the new copy.
// ROWS (team size a multiple of n): every element a thread owns has the same row
// r = rank mod n, so the thread reads that row of each factor into registers once per
// mode instead of once per element.
template <typename T, typename TO, int NN, int EMAX, bool DET, bool ROWS = false>
__device__ __forceinline__ void gq_entry_elem(const T *const *mats, const T *const *in, TO *const *out, int d,
                                              int stride, int N, long long e, T *buf, T *buf2, T *fac, T *acc,
                                              T *part, bool first, bool last, const Team &tm)
{
    constexpr int P = NN * NN;
    const int F = N / NN;
    const int r0 = tm.rank % NN;
    tm.sync();
    stage_vector(buf, in[e], N, tm);
    stage_factors<T, NN>(fac, mats + e * d, d, stride, tm);
    tm.sync();
    TO *o = out[e];
    const T *src = buf;
    T *dst = buf2;
    for (int i = d - 1; i >= 0; --i) {
        const T *M = fac + i * P;
        T mrow[NN];
        if constexpr (ROWS) {
#pragma unroll
            for (int k = 0; k < NN; ++k) mrow[k] = M[r0 + k * NN];
        }
#pragma unroll
        for (int j = 0; j < EMAX; ++j) {
            const int q = tm.rank + j * tm.size;
            if (q < N) {
                const int c = q / NN, r = ROWS ? r0 : q - c * NN;
                T x[NN];
                load_fibre<T, NN>(src + c * NN, x);
                T s = T(0);
#pragma unroll
                for (int k = 0; k < NN; ++k) s = fma_t<T>(ROWS ? mrow[k] : M[r + k * NN], x[k], s);
                if (i > 0)
                    dst[c + r * F] = s;
                else
                    gq_add<T, TO, DET>(o, acc, part, c + r * F, s, first, last);
            }
        }
        if (i > 0) {
            tm.sync();  // the mode's results are complete in dst, its reads of src done
            T *t = const_cast<T *>(src);
            src = dst;
            dst = t;
        }
    }
}

// Atomic mode: every entry added into its output with atomics as soon as it is
// computed.  Deterministic mode: entries in sorted order, runs of one output summed
// in a shared-memory accumulator (team_elems covers it) and added once.  No run sums
// in registers: the register footprint of the single-call kernels, 3 FP64 / 4 FP32
// CTAs of 256 threads per SM.
// Run edges of entry ei in unit [b, e) (deterministic mode): whether it starts / ends
// a run of equal output pointers within the unit, and at a run's last entry the
// partial slot its sum goes to (null: the run is a whole segment, added directly).
template <typename T, bool DET>
__device__ __forceinline__ T *gq_run_edges(const GqArgs &a, long long b, long long e, long long ei, long long &rs,
                                           bool &first, bool &last)
{
    if constexpr (DET) {
        const unsigned long long *k = a.keys;
        first = ei == b || k[ei - 1] != k[ei];
        last = ei + 1 == e || k[ei + 1] != k[ei];
        if (first) rs = ei;
        if (!last) return nullptr;
        const bool from_prev = rs == b && b > 0 && k[b - 1] == k[b];
        const bool into_next = ei + 1 == e && e < a.nb && k[e] == k[ei];
        if (!from_prev && !into_next) return nullptr;
        const long long slot = 2 * (b / a.unit) + (from_prev ? 0 : 1);
        return reinterpret_cast<T *>(a.partial) + slot * (long long)a.N;
    } else {
        first = last = true;
        return nullptr;
    }
}

template <typename T, typename TO, int NN, int QMAX, bool DET>
__global__ void __launch_bounds__(kGroupedBlock, sizeof(T) == 8 ? 3 : 4) gq_fibre_kernel(const GqArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_unit[kGroupedBlock / 8];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    T *acc = buf + (a.team_elems - a.vec_pad);  // deterministic mode: the slice's last vec_pad values
    const T *const *mats = reinterpret_cast<const T *const *>(a.mats);
    const T *const *in = reinterpret_cast<const T *const *>(a.in);
    TO *const *out = reinterpret_cast<TO *const *>(a.out);
    long long b, e;
    unsigned claim = gq_first_claim(a, tm);
    while (gq_next(a, &s_unit[tm.id], tm, claim, b, e))
    {
        long long rs = b;
        for (long long ei = b; ei < e; ++ei) {
            bool first, last;
            T *part = gq_run_edges<T, DET>(a, b, e, ei, rs, first, last);
            gq_entry_fibre<T, TO, NN, QMAX, DET>(mats, in, out, a.d, a.stride, a.N, ei, buf, fac, acc, part, first,
                                                 last, tm);
        }
    }
}

// FP64 atomic mode with at most 4 outputs per thread fits 48 registers without spills:
// 5 CTAs of 256 threads per SM (more warps to keep the FP64 pipe fed across barriers);
// the rows form holds n more values and gets 64 registers (4 CTAs).
template <typename T, typename TO, int NN, int EMAX, bool DET, bool ROWS = false>
__global__ void __launch_bounds__(kGroupedBlock, sizeof(T) == 8 ? (DET || EMAX > 4 ? 3 : (ROWS ? 4 : 5)) : 4)
    gq_elem_kernel(const GqArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_unit[kGroupedBlock / 8];
    const Team tm(a.team_size);
    // slice: [vector | second vector | factors | run sums (deterministic mode)]
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *buf2 = buf + a.vec_pad;
    T *fac = buf + 2 * a.vec_pad;
    T *acc = buf + (a.team_elems - a.vec_pad);
    const T *const *mats = reinterpret_cast<const T *const *>(a.mats);
    const T *const *in = reinterpret_cast<const T *const *>(a.in);
    TO *const *out = reinterpret_cast<TO *const *>(a.out);
    long long b, e;
    unsigned claim = gq_first_claim(a, tm);
    while (gq_next(a, &s_unit[tm.id], tm, claim, b, e))
    {
        long long rs = b;
        for (long long ei = b; ei < e; ++ei) {
            bool first, last;
            T *part = gq_run_edges<T, DET>(a, b, e, ei, rs, first, last);
            gq_entry_elem<T, TO, NN, EMAX, DET, ROWS>(mats, in, out, a.d, a.stride, a.N, ei, buf, buf2, fac, acc,
                                                      part, first, last, tm);
        }
    }
}

// n = 9..16: element mapping with n at run time
template <typename T, typename TO, int EMAX, bool DET>
__global__ void __launch_bounds__(kGroupedBlock, 2) gq_elem_rt_kernel(const GqArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_unit[kGroupedBlock / 8];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    const T *const *mats = reinterpret_cast<const T *const *>(a.mats);
    const T *const *in = reinterpret_cast<const T *const *>(a.in);
    TO *const *out = reinterpret_cast<TO *const *>(a.out);
    long long b, e;
    unsigned claim = gq_first_claim(a, tm);
    while (gq_next(a, &s_unit[tm.id], tm, claim, b, e))
        team_forward_elem<T, TO, EMAX, DET>(mats, in, out, nullptr, a.d, a.n, a.stride, a.N, b, e, buf, fac, tm);
}

}  // namespace kgb

// Lookups of every instantiation for one (T, TO) = (KGB_T, KGB_TO), defined by the
// including translation unit.  Fibre kernels: QMAX up to 8 for n <= 4, up to 4 above
// (the planner's cap).  Element kernels with compile-time n: FP64 only (where the
// pipe is charged per warp instruction, so idle lanes cost time).
#define KGB_GQ_F1(NN, Q)                                                                                   \
    case NN * 32 + Q * 2: return gq_fibre_kernel<KGB_T, KGB_TO, NN, Q, false>;                             \
    case NN * 32 + Q * 2 + 1: return gq_fibre_kernel<KGB_T, KGB_TO, NN, Q, true>;
#define KGB_GQ_FS(NN) KGB_GQ_F1(NN, 1) KGB_GQ_F1(NN, 2) KGB_GQ_F1(NN, 4) KGB_GQ_F1(NN, 8)
#define KGB_GQ_FL(NN) KGB_GQ_F1(NN, 1) KGB_GQ_F1(NN, 2) KGB_GQ_F1(NN, 4)
#define KGB_GQ_E1(NN, E)                                                                                   \
    case NN * 32 + E * 2: return gq_elem_kernel<KGB_T, KGB_TO, NN, E, false>;                              \
    case NN * 32 + E * 2 + 1: return gq_elem_kernel<KGB_T, KGB_TO, NN, E, true>;
#define KGB_GQ_E(NN) KGB_GQ_E1(NN, 1) KGB_GQ_E1(NN, 2) KGB_GQ_E1(NN, 4) KGB_GQ_E1(NN, 8)
#define KGB_GQ_ER1(NN, E)                                                                                  \
    case NN * 32 + E * 2: return gq_elem_kernel<KGB_T, KGB_TO, NN, E, false, true>;                        \
    case NN * 32 + E * 2 + 1: return gq_elem_kernel<KGB_T, KGB_TO, NN, E, true, true>;
#define KGB_GQ_ER(NN) KGB_GQ_ER1(NN, 2) KGB_GQ_ER1(NN, 4)
#define KGB_GQ_R(E)                                                                                        \
    case E * 2: return gq_elem_rt_kernel<KGB_T, KGB_TO, E, false>;                                         \
    case E * 2 + 1: return gq_elem_rt_kernel<KGB_T, KGB_TO, E, true>;

#define KGB_GQ_LOOKUP_FIBRE_AND_RT                                                                         \
    template <> GqFn gq_fibre_lookup<KGB_T, KGB_TO>(int nn, int qmax, bool det)                            \
    {                                                                                                      \
        switch (nn * 32 + qmax * 2 + (det ? 1 : 0)) {                                                      \
            KGB_GQ_FS(2) KGB_GQ_FS(3) KGB_GQ_FS(4) KGB_GQ_FL(5) KGB_GQ_FL(6) KGB_GQ_FL(7) KGB_GQ_FL(8)      \
        default: return nullptr;                                                                           \
        }                                                                                                  \
    }                                                                                                      \
    template <> GqFn gq_elem_rt_lookup<KGB_T, KGB_TO>(int emax, bool det)                                  \
    {                                                                                                      \
        switch (emax * 2 + (det ? 1 : 0)) {                                                                \
            KGB_GQ_R(1) KGB_GQ_R(2) KGB_GQ_R(4) KGB_GQ_R(8) KGB_GQ_R(16)                                    \
        default: return nullptr;                                                                           \
        }                                                                                                  \
    }
#define KGB_GQ_LOOKUP_ELEM                                                                                 \
    template <> GqFn gq_elem_lookup<KGB_T, KGB_TO>(int nn, int emax, bool det)                             \
    {                                                                                                      \
        switch (nn * 32 + emax * 2 + (det ? 1 : 0)) {                                                      \
            KGB_GQ_E(2) KGB_GQ_E(3) KGB_GQ_E(4) KGB_GQ_E(5) KGB_GQ_E(6) KGB_GQ_E(7) KGB_GQ_E(8)             \
        default: return nullptr;                                                                           \
        }                                                                                                  \
    }                                                                                                      \
    template <> GqFn gq_elem_rows_lookup<KGB_T, KGB_TO>(int nn, int emax, bool det)                        \
    {                                                                                                      \
        switch (nn * 32 + emax * 2 + (det ? 1 : 0)) {                                                      \
            KGB_GQ_ER(4) KGB_GQ_ER(8)                                                                      \
        default: return nullptr;                                                                           \
        }                                                                                                  \
    }
#define KGB_GQ_LOOKUP_NO_ELEM                                                                              \
    template <> GqFn gq_elem_lookup<KGB_T, KGB_TO>(int, int, bool) { return nullptr; }                     \
    template <> GqFn gq_elem_rows_lookup<KGB_T, KGB_TO>(int, int, bool) { return nullptr; }
