// Forward kernels: output[k] += kron(A_{k,0..d-1}) . input[k].
//
// Replaces the reference's one-CTA-per-entry kernel that ping-pongs through the
// caller's global `input`/`workspace` vectors (kronmult_gpu/kronmult.cu:95-167).
// Here each entry's N-vector and its d factors are staged in shared memory once,
// the d mode products of the backward Algorithm-993 sweep run in place in that
// buffer through registers, and consecutive entries that target the same output
// vector are summed in registers before one atomic add per element.
//
// Mode product (kronmult_gpu/kronmult.cu:54-78): with X the current vector seen
// as an n x F col-major matrix (F = N/n fibres of n contiguous values),
//     Y[c + r*F] = sum_{k=0..n-1} A_i(r, k) * X[k + c*n]
// summed k-ascending from 0 with fused multiply-adds, exactly as the reference
// kernel's `dotprod += X * Mt` does.  Modes run i = d-1 .. 0; after d steps the
// index rotation returns the vector to its natural order.
#pragma once
#include "common.cuh"

namespace kgb {

template <typename T, typename TO> struct FwdArgs {
    const T *const *mats;  // nb*d factor pointers, entry k's factors at [k*d, k*d+d)
    const T *const *in;    // nb input pointers (N values each)
    TO *const *out;        // nb output pointers (may alias)
    T *const *ws;          // nb workspace pointers (global-memory paths only; may be null)
    long long nb;          // number of entries
    int d, n, stride;      // factor count, factor size, factor leading dimension
    int N;                 // n^d
    int team_size;         // threads per team
    int teams_per_cta;     // teams in one CTA
    int entries_per_team;  // contiguous entries each team processes
    int team_elems;        // shared-memory elements reserved per team
    int vec_pad;           // offset of the factor area inside a team's slice (elements)
    int fac_pad;           // padded size of the factor area (elements)
    int prefetch;          // 1: two staging slots per team, next entry copied asynchronously
    // two-pass path for vectors beyond shared memory (split_pass1/2_kernel):
    int split_d1;          // fast modes run by pass 1 (d-1 .. d-split_d1)
    int split_C;           // n^split_d1: chunk of contiguous values pass 1 sweeps
    int split_R;           // n^(d-split_d1): values sharing a fast position (stride split_C)
    int split_L;           // fast positions per pass-2 tile
    int split_ept1;        // chunks each pass-1 team sweeps (the next one copied while computing)
};

// ---- helpers ---------------------------------------------------------------

// copy N values of an input vector into shared memory, 16-byte vectors when the
// source is 16-byte aligned and N*sizeof(T) is a multiple of 16
// ---- swizzled vector layout ------------------------------------------------
// Fibres of 32 bytes (two 16-byte chunks) read by consecutive lanes would put two
// lanes of a quarter-warp on the same banks.  FP32 vectors with n = 8 are staged
// with 16-byte chunk ch stored at chunk ch ^ ((ch >> 3) & 7): the chunks one
// quarter-warp reads then land on distinct banks, and each aligned group of 8
// chunks (one 128-byte row) is only permuted within itself, so stores of
// consecutive elements stay conflict-free.  (FP64 kernels are bound by the FP64
// pipe, not by shared memory, and keep the plain layout and its lower register
// count.)
template <typename T, int NN> struct VecSwizzle {
    static constexpr bool on = sizeof(T) == 4 && NN * sizeof(T) == 32;
};

__device__ __forceinline__ int swz_chunk(int ch) { return ch ^ ((ch >> 3) & 7); }

// shared-memory position of vector element e
template <typename T, bool SWZ> __device__ __forceinline__ int vec_pos(int e)
{
    if constexpr (SWZ) {
        constexpr int per = 16 / (int)sizeof(T);
        return swz_chunk(e / per) * per + (e & (per - 1));
    } else {
        return e;
    }
}

template <typename T, bool SWZ = false>
__device__ __forceinline__ void stage_vector(T *dst, const T *src, int N, const Team &tm)
{
    const size_t bytes = (size_t)N * sizeof(T);
    if (((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && ((bytes & 15u) == 0)) {
        const int nv = (int)(bytes >> 4);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        for (int v = tm.rank; v < nv; v += tm.size) d4[SWZ ? swz_chunk(v) : v] = __ldcs(s4 + v);
    } else {
        for (int v = tm.rank; v < N; v += tm.size) dst[vec_pos<T, SWZ>(v)] = __ldcs(src + v);
    }
}

// copy the d factors of an entry into shared memory as fac[i*n*n + r + k*n] = A_i(r,k)
template <typename T, int NN>
__device__ __forceinline__ void stage_factors(T *fac, const T *const *mats, int d, int stride, const Team &tm)
{
    constexpr int NN2 = NN * NN;
    for (int idx = tm.rank; idx < d * NN2; idx += tm.size) {
        const int i = idx / NN2;
        const int rem = idx - i * NN2;
        const int k = rem / NN;
        const int r = rem - k * NN;
        fac[idx] = mats[i][r + (size_t)k * stride];
    }
}

// bytes of the widest aligned vector load for one fibre of NN values of type T
template <typename T, int NN> struct FibreVec {
    static constexpr int bytes = NN * (int)sizeof(T);
    static constexpr int width = (bytes % 16 == 0) ? 16 : (bytes % 8 == 0) ? 8 : (int)sizeof(T);
};

template <typename T, int NN> __device__ __forceinline__ void load_fibre(const T *p, T (&x)[NN])
{
    constexpr int W = FibreVec<T, NN>::width;
    if constexpr (W == 16) {
        const int4 *p4 = reinterpret_cast<const int4 *>(p);
#pragma unroll
        for (int v = 0; v < (int)(NN * sizeof(T) / 16); ++v) {
            int4 t = p4[v];
            *reinterpret_cast<int4 *>(&x[v * 16 / sizeof(T)]) = t;
        }
    } else if constexpr (W == 8 && sizeof(T) == 4) {
        const float2 *p2 = reinterpret_cast<const float2 *>(p);
#pragma unroll
        for (int v = 0; v < NN / 2; ++v) {
            float2 t = p2[v];
            x[2 * v] = t.x;
            x[2 * v + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < NN; ++k) x[k] = p[k];
    }
}

// Packed FP32 pairs (sm_100 family: add / sub / mul / fma .rn.f32x2): two independent
// lanes per instruction, each rounded exactly as the scalar operation (the FP32 pipe's
// rate is unchanged; the instructions to issue are halved).
using f2 = unsigned long long;
__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 f2_neg(f2 a) { return a ^ 0x8000000080000000ull; }

template <typename T> __device__ __forceinline__ T fma_t(T a, T b, T c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Factors too large to keep in registers (NN*NN*sizeof(T) > 128 bytes).
template <typename T, int NN> struct FactorInSmem {
    static constexpr bool value = NN * NN * sizeof(T) > 128;
};

// y[r] = sum_k M(r, k) * x[k] for one fibre, M col-major NN x NN in shared memory.
// Column k is fetched with the widest aligned vector load (the layout keeps every
// factor 16-byte aligned and a column's offset a multiple of the fibre load width)
// and feeds all NN rows, so one broadcast load serves up to 16/sizeof(T) x NN FMAs
// instead of one.  Each y[r] is still the k-ascending FMA chain from 0.
template <typename T, int NN>
__device__ __forceinline__ void mode_fibre_smem(const T *M, const T (&xv)[NN], T (&y)[NN])
{
#pragma unroll
    for (int r = 0; r < NN; ++r) y[r] = T(0);
#pragma unroll
    for (int k = 0; k < NN; ++k) {
        T col[NN];
        load_fibre<T, NN>(M + k * NN, col);
#pragma unroll
        for (int r = 0; r < NN; ++r) y[r] = fma_t<T>(col[r], xv[k], y[r]);
    }
}

// The same for two fibres at once: each column load feeds 2 x NN FMAs.
template <typename T, int NN>
__device__ __forceinline__ void mode_fibre2_smem(const T *M, const T (&x0)[NN], const T (&x1)[NN], T (&y0)[NN],
                                                 T (&y1)[NN])
{
#pragma unroll
    for (int r = 0; r < NN; ++r) {
        y0[r] = T(0);
        y1[r] = T(0);
    }
#pragma unroll
    for (int k = 0; k < NN; ++k) {
        T col[NN];
        load_fibre<T, NN>(M + k * NN, col);
#pragma unroll
        for (int r = 0; r < NN; ++r) {
            y0[r] = fma_t<T>(col[r], x0[k], y0[r]);
            y1[r] = fma_t<T>(col[r], x1[k], y1[r]);
        }
    }
}

// fibre c (NN values from element c*NN) of a staged vector, swizzled or not
template <typename T, int NN, bool SWZ>
__device__ __forceinline__ void load_fibre_v(const T *buf, int c, T (&x)[NN])
{
    if constexpr (SWZ) {
        constexpr int P = NN * (int)sizeof(T) / 16;
        const int4 *b4 = reinterpret_cast<const int4 *>(buf);
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const int4 t = b4[swz_chunk(c * P + j)];
            *reinterpret_cast<int4 *>(&x[j * 16 / (int)sizeof(T)]) = t;
        }
    } else {
        load_fibre<T, NN>(buf + c * NN, x);
    }
}

// One mode product of a team over its fibres c = rank + q*size < F (q < QMAX):
// y[q] = M . fibre c.  Factors held in registers (m) are used directly; factors in
// shared memory are read a column at a time, shared by pairs of fibres.
template <typename T, int NN, int QMAX, bool SWZ, bool REGM>
__device__ __forceinline__ void mode_team(const T *buf, const T *M, const T *m, int F, const Team &tm,
                                          T (&y)[QMAX][NN])
{
    if constexpr (REGM) {
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int c = tm.rank + q * tm.size;
            if (c < F) {
                T xv[NN];
                load_fibre_v<T, NN, SWZ>(buf, c, xv);
#pragma unroll
                for (int r = 0; r < NN; ++r) {
                    T s = T(0);
#pragma unroll
                    for (int k = 0; k < NN; ++k) s = fma_t<T>(m[r + k * NN], xv[k], s);
                    y[q][r] = s;
                }
            }
        }
    } else {
        // highest rank in this thread's warp (teams of fewer than 32 threads share a
        // warp with other teams of the same size), so that the pair / single choice
        // below is uniform across the warp
        const int last = tm.size < 32 ? tm.size - 1 : (tm.rank | 31);
#pragma unroll
        for (int q = 0; q < QMAX; q += 2) {
            const int c0 = tm.rank + q * tm.size;
            if constexpr (QMAX >= 2) {
                if (last + (q + 1) * tm.size < F) {
                    T x0[NN], x1[NN];
                    load_fibre_v<T, NN, SWZ>(buf, c0, x0);
                    load_fibre_v<T, NN, SWZ>(buf, c0 + tm.size, x1);
                    mode_fibre2_smem<T, NN>(M, x0, x1, y[q], y[q + 1]);
                    continue;
                }
            }
#pragma unroll
            for (int h = 0; h < (QMAX >= 2 ? 2 : 1); ++h) {
                const int c = c0 + h * tm.size;
                if (c < F) {
                    T x0[NN];
                    load_fibre_v<T, NN, SWZ>(buf, c, x0);
                    mode_fibre_smem<T, NN>(M, x0, y[q + h]);
                }
            }
        }
    }
}

// ---- asynchronous global->shared copies (cp.async, completion per thread) --

template <int BYTES> __device__ __forceinline__ void cp_async(void *dst, const void *src)
{
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    if constexpr (BYTES == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(src), "n"(BYTES) : "memory");
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// issue the copies of one entry's input vector and factors into a staging slot
// (same layouts as stage_vector / stage_factors); completes with cp_async_wait_all
template <typename T, int NN, bool SWZ = false>
__device__ __forceinline__ void stage_async(T *dst, T *fac, const T *src, const T *const *mats, int N, int d,
                                            int stride, const Team &tm)
{
    const size_t bytes = (size_t)N * sizeof(T);
    if (((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && ((bytes & 15u) == 0)) {
        const int nv = (int)(bytes >> 4);
        for (int v = tm.rank; v < nv; v += tm.size)
            cp_async<16>(reinterpret_cast<int4 *>(dst) + (SWZ ? swz_chunk(v) : v),
                         reinterpret_cast<const int4 *>(src) + v);
    } else {
        for (int v = tm.rank; v < N; v += tm.size) cp_async<(int)sizeof(T)>(dst + vec_pos<T, SWZ>(v), src + v);
    }
    constexpr int NN2 = NN * NN;
    for (int idx = tm.rank; idx < d * NN2; idx += tm.size) {
        const int i = idx / NN2;
        const int rem = idx - i * NN2;
        const int k = rem / NN;
        const int r = rem - k * NN;
        cp_async<(int)sizeof(T)>(fac + idx, mats[i] + r + (size_t)k * stride);
    }
    cp_async_commit();
}

// ---- shared-memory, register in-place team forward (compile-time n) -------
//
// Thread `rank` of a team owns fibres c = rank + q*team_size (q < QMAX) in every
// mode and computes all n outputs of each of its fibres, so each staged input
// value is read from shared memory once per mode.  The mode is done in place:
// every thread reads its fibres into registers, the team synchronises, and the
// results are written to their rotated positions c + r*F.
//
// The team walks entries [e_begin, e_end) (through `perm` when given) and sums
// consecutive entries with the same output pointer in registers.  A run is
// flushed with atomic adds, or -- in deterministic mode, where the caller
// guarantees that every output pointer is one contiguous run owned by this team --
// with a plain read-modify-write, so that the sum order is the entry order.
template <typename T, typename TO, int NN, int QMAX, bool DET, bool PF = false>
__device__ __forceinline__ void team_forward(const T *const *mats, const T *const *in, TO *const *out,
                                             const long long *perm, int d, int stride, int N, long long e_begin,
                                             long long e_end, T *buf, T *fac, const Team &tm, T *buf2 = nullptr,
                                             T *fac2 = nullptr)
{
    // PF: two staging slots (buf/fac and buf2/fac2); the copies of entry e+1 are in
    // flight (cp.async) while entry e is computed
    const int F = N / NN;
    // a run of entries is summed in the compute type (FP32 accumulation for FP32
    // storage); the output type is used only for the final addition into the output
    T acc[QMAX][NN];
    TO *cur = nullptr;

    auto flush = [&](TO *dst) {
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int c = tm.rank + q * tm.size;
            if (c < F) {
#pragma unroll
                for (int r = 0; r < NN; ++r) {
                    if constexpr (DET) {
                        dst[c + r * F] = dst[c + r * F] + (TO)acc[q][r];
                    } else {
                        atomic_add<TO>(dst + c + r * F, (TO)acc[q][r]);
                    }
                }
            }
        }
    };

    constexpr bool kSwz = VecSwizzle<T, NN>::on;
    if constexpr (PF) {
        if (e_begin < e_end) {
            const long long e0 = perm ? perm[e_begin] : e_begin;
            stage_async<T, NN, kSwz>(buf, fac, in[e0], mats + e0 * d, N, d, stride, tm);
        }
    }
    for (long long ei = e_begin; ei < e_end; ++ei) {
        const long long e = perm ? perm[ei] : ei;
        TO *o = out[e];
        if constexpr (PF) {
            cp_async_wait_all();
            tm.sync();  // slot of entry e complete for the whole team
            if (ei + 1 < e_end) {
                const long long en = perm ? perm[ei + 1] : ei + 1;
                stage_async<T, NN, kSwz>(buf2, fac2, in[en], mats + en * d, N, d, stride, tm);
            }
        } else {
            stage_vector<T, kSwz>(buf, in[e], N, tm);
            stage_factors<T, NN>(fac, mats + e * d, d, stride, tm);
            tm.sync();
        }

        T y[QMAX][NN];
        for (int i = d - 1; i >= 0; --i) {
            const T *M = fac + i * NN * NN;
            // small factors are held in registers; larger ones are read from shared
            // memory, where every lane of a warp reads the same address (broadcast)
            constexpr bool kRegM = !FactorInSmem<T, NN>::value;
            T m[kRegM ? NN * NN : 1];
            if constexpr (kRegM) {
#pragma unroll
                for (int j = 0; j < NN * NN; ++j) m[j] = M[j];
            }
            mode_team<T, NN, QMAX, kSwz, kRegM>(buf, M, m, F, tm, y);
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
        // y[q][r] is element c + r*F of kron(A) . x
        if (o != cur) {
            if (cur != nullptr) flush(cur);
            cur = o;
#pragma unroll
            for (int q = 0; q < QMAX; ++q)
#pragma unroll
                for (int r = 0; r < NN; ++r) acc[q][r] = y[q][r];
        } else {
#pragma unroll
            for (int q = 0; q < QMAX; ++q)
#pragma unroll
                for (int r = 0; r < NN; ++r) acc[q][r] += y[q][r];
        }
        if constexpr (PF) {
            T *t = buf;
            buf = buf2;
            buf2 = t;
            t = fac;
            fac = fac2;
            fac2 = t;
        }
    }
    if (cur != nullptr) flush(cur);
}

// Ping-pong variant of team_forward (same run / deterministic semantics) for
// factors read from shared memory: every mode reads one vector buffer and writes
// the other, so a thread stores each output fibre as soon as it is computed -- one
// barrier per mode instead of two, and no register array of all of the thread's
// mode outputs besides the run sums.  Three vector buffers: the two of the entry
// being computed and the one the next entry streams into (cp.async).
template <typename T, typename TO, int NN, int QMAX, bool DET>
__device__ __forceinline__ void team_forward_pp(const T *const *mats, const T *const *in, TO *const *out, int d,
                                                int stride, int N, long long e_begin, long long e_end, T *vb0,
                                                T *vb1, T *vb2, T *fb0, T *fb1, const Team &tm)
{
    const int F = N / NN;
    constexpr bool kSwz = VecSwizzle<T, NN>::on;
    T acc[QMAX][NN];
    TO *cur = nullptr;
    auto flush = [&](TO *dst) {
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int c = tm.rank + q * tm.size;
            if (c < F) {
#pragma unroll
                for (int r = 0; r < NN; ++r) {
                    if constexpr (DET) {
                        dst[c + r * F] = dst[c + r * F] + (TO)acc[q][r];
                    } else {
                        atomic_add<TO>(dst + c + r * F, (TO)acc[q][r]);
                    }
                }
            }
        }
    };
    T *vcur = vb0, *vpp = vb1, *vnxt = vb2;
    T *fcur = fb0, *fnxt = fb1;
    if (e_begin < e_end) stage_async<T, NN, kSwz>(vcur, fcur, in[e_begin], mats + e_begin * d, N, d, stride, tm);
    // highest rank in this thread's warp: the pair / single choice below is warp-uniform
    const int last = tm.size < 32 ? tm.size - 1 : (tm.rank | 31);
    for (long long e = e_begin; e < e_end; ++e) {
        TO *o = out[e];
        cp_async_wait_all();
        tm.sync();  // entry e staged for the whole team; entry e-1 done with every buffer
        if (e + 1 < e_end)
            stage_async<T, NN, kSwz>(vnxt, fnxt, in[e + 1], mats + (e + 1) * d, N, d, stride, tm);
        const bool fresh = o != cur;
        if (fresh) {
            if (cur != nullptr) flush(cur);
            cur = o;
        }
        const T *src = vcur;
        T *dst = vpp;
        for (int i = d - 1; i >= 0; --i) {
            const T *M = fcur + i * NN * NN;
#pragma unroll
            for (int q = 0; q < QMAX; q += 2) {
                const int c0 = tm.rank + q * tm.size;
                bool pair = false;
                if constexpr (QMAX >= 2) pair = last + (q + 1) * tm.size < F;
                if (pair) {
                    if constexpr (QMAX >= 2) {
                        T x0[NN], x1[NN], y0[NN], y1[NN];
                        load_fibre_v<T, NN, kSwz>(src, c0, x0);
                        load_fibre_v<T, NN, kSwz>(src, c0 + tm.size, x1);
                        mode_fibre2_smem<T, NN>(M, x0, x1, y0, y1);
                        if (i > 0) {
#pragma unroll
                            for (int r = 0; r < NN; ++r) {
                                dst[vec_pos<T, kSwz>(c0 + r * F)] = y0[r];
                                dst[vec_pos<T, kSwz>(c0 + tm.size + r * F)] = y1[r];
                            }
                        } else {
#pragma unroll
                            for (int r = 0; r < NN; ++r) {
                                acc[q][r] = fresh ? y0[r] : acc[q][r] + y0[r];
                                acc[q + 1][r] = fresh ? y1[r] : acc[q + 1][r] + y1[r];
                            }
                        }
                    }
                } else {
#pragma unroll
                    for (int h = 0; h < (QMAX >= 2 ? 2 : 1); ++h) {
                        const int c = c0 + h * tm.size;
                        if (c < F) {
                            T x0[NN], y0[NN];
                            load_fibre_v<T, NN, kSwz>(src, c, x0);
                            mode_fibre_smem<T, NN>(M, x0, y0);
                            if (i > 0) {
#pragma unroll
                                for (int r = 0; r < NN; ++r) dst[vec_pos<T, kSwz>(c + r * F)] = y0[r];
                            } else {
#pragma unroll
                                for (int r = 0; r < NN; ++r)
                                    acc[q + h][r] = fresh ? y0[r] : acc[q + h][r] + y0[r];
                            }
                        }
                    }
                }
            }
            if (i > 0) {
                tm.sync();  // mode outputs complete; every read of src done
                T *t = const_cast<T *>(src);
                src = dst;
                dst = t;
            }
        }
        T *t = vcur;  // the next entry's buffer becomes current; the old one is the next target
        vcur = vnxt;
        vnxt = t;
        t = fcur;
        fcur = fnxt;
        fnxt = t;
    }
    if (cur != nullptr) flush(cur);
    cp_async_wait_all();
}

// FP32 variants are capped at 64 registers so that four 256-thread CTAs fit on an SM
// Element-mapped team forward with run accumulation (runtime n): thread `rank`
// owns output elements q = rank + j*team_size (j < EMAX) of every mode, so all lanes
// have work for any (d, n).  Element q is row r = q % n of fibre c = q / n: lanes that
// share a fibre read the same shared-memory words (broadcast), and only the one store
// per output, to position c + r*F, is strided.  Same run / deterministic semantics as
// team_forward.
template <typename T, typename TO, int EMAX, bool DET>
__device__ __forceinline__ void team_forward_elem(const T *const *mats, const T *const *in, TO *const *out,
                                                  const long long *perm, int d, int n, int stride, int N,
                                                  long long e_begin, long long e_end, T *buf, T *fac,
                                                  const Team &tm)
{
    const int F = N / n, P = n * n;
    T acc[EMAX];
    TO *cur = nullptr;
    auto flush = [&](TO *dst) {
#pragma unroll
        for (int j = 0; j < EMAX; ++j) {
            const int q = tm.rank + j * tm.size;
            if (q < N) {
                const int c = q / n, r = q - c * n, p = c + r * F;
                if constexpr (DET) {
                    dst[p] = dst[p] + (TO)acc[j];
                } else {
                    atomic_add<TO>(dst + p, (TO)acc[j]);
                }
            }
        }
    };
    for (long long ei = e_begin; ei < e_end; ++ei) {
        const long long e = perm ? perm[ei] : ei;
        TO *o = out[e];
        stage_vector(buf, in[e], N, tm);
        {
            const T *const *m = mats + e * d;
            for (int idx = tm.rank; idx < d * P; idx += tm.size) {
                const int i = idx / P, rem = idx - i * P, k = rem / n, r = rem - k * n;
                fac[idx] = m[i][r + (size_t)k * stride];
            }
        }
        tm.sync();
        T y[EMAX];
        for (int i = d - 1; i >= 0; --i) {
            const T *M = fac + i * P;
#pragma unroll
            for (int j = 0; j < EMAX; ++j) {
                const int q = tm.rank + j * tm.size;
                if (q < N) {
                    const int c = q / n, r = q - c * n;
                    const T *x = buf + c * n;
                    T s = T(0);
#pragma unroll 8
                    for (int k = 0; k < n; ++k) s = fma_t<T>(M[r + k * n], x[k], s);
                    y[j] = s;
                }
            }
            tm.sync();  // every read of buf (and fac) for this mode is done
            if (i > 0) {
#pragma unroll
                for (int j = 0; j < EMAX; ++j) {
                    const int q = tm.rank + j * tm.size;
                    if (q < N) {
                        const int c = q / n, r = q - c * n;
                        buf[c + r * F] = y[j];
                    }
                }
                tm.sync();
            }
        }
        if (o != cur) {
            if (cur != nullptr) flush(cur);
            cur = o;
#pragma unroll
            for (int j = 0; j < EMAX; ++j) acc[j] = y[j];
        } else {
#pragma unroll
            for (int j = 0; j < EMAX; ++j) acc[j] += y[j];
        }
    }
    if (cur != nullptr) flush(cur);
}

// Element-mapped team forward with a fully asynchronous two-slot pipeline: while
// entry e is computed, the copies of entry e+1's vector and factors are in flight
// (cp.async), issued from pointers that were themselves copied into shared memory
// (cp.async) one entry earlier, so no dependent global load sits on the critical
// path.  Slot layout per team: [vec A][fac A][vec B][fac B][ptr A][ptr B] where a
// pointer slot holds the entry's input pointer and its d factor pointers.
template <typename T>
__device__ __forceinline__ void elem_copy_ptrs(const T **pslot, const T *const *in, const T *const *mats,
                                               long long e, int d, const Team &tm)
{
    for (int v = tm.rank; v <= d; v += tm.size) {
        const void *src = v == 0 ? (const void *)(in + e) : (const void *)(mats + e * d + (v - 1));
        cp_async<8>(pslot + v, src);
    }
}

template <typename T>
__device__ __forceinline__ void elem_copy_data(T *vec, T *fac, const T *const *pslot, int d, int n, int stride,
                                               int N, const Team &tm)
{
    const T *src = pslot[0];
    const size_t bytes = (size_t)N * sizeof(T);
    if (((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && ((bytes & 15u) == 0)) {
        for (int v = tm.rank; v < (int)(bytes >> 4); v += tm.size)
            cp_async<16>(reinterpret_cast<int4 *>(vec) + v, reinterpret_cast<const int4 *>(src) + v);
    } else {
        for (int v = tm.rank; v < N; v += tm.size) cp_async<(int)sizeof(T)>(vec + v, src + v);
    }
    const int P = n * n;
    for (int idx = tm.rank; idx < d * P; idx += tm.size) {
        const int i = idx / P, rem = idx - i * P, k = rem / n, r = rem - k * n;
        cp_async<(int)sizeof(T)>(fac + idx, pslot[1 + i] + r + (size_t)k * stride);
    }
}

template <typename T, typename TO, int EMAX, bool DET>
__device__ __forceinline__ void team_forward_elem_pf(const T *const *mats, const T *const *in, TO *const *out,
                                                     const long long *perm, int d, int n, int stride, int N,
                                                     long long e_begin, long long e_end, T *slots, int slot_elems,
                                                     const T **ptrs, const Team &tm)
{
    if (e_begin >= e_end) return;
    const int F = N / n, P = n * n;
    constexpr int kAlign = 16 / (int)sizeof(T);
    const int vpad = (N + kAlign - 1) / kAlign * kAlign;  // factors follow the vector in a slot
    auto vec = [&](int s) { return s ? slots + slot_elems : slots; };
    auto fac = [&](int s) { return (s ? slots + slot_elems : slots) + vpad; };
    auto pslot = [&](int s) { return s ? ptrs + (d + 1) : ptrs; };
    auto entry = [&](long long ei) { return perm ? perm[ei] : ei; };

    T acc[EMAX];
    TO *cur = nullptr;
    auto flush = [&](TO *dst) {
#pragma unroll
        for (int j = 0; j < EMAX; ++j) {
            const int q = tm.rank + j * tm.size;
            if (q < N) {
                const int c = q / n, r = q - c * n, p = c + r * F;
                if constexpr (DET) {
                    dst[p] = dst[p] + (TO)acc[j];
                } else {
                    atomic_add<TO>(dst + p, (TO)acc[j]);
                }
            }
        }
    };

    // prologue: pointers of the first entry (waited for), its data copy, pointers of the second
    elem_copy_ptrs<T>(pslot(0), in, mats, entry(e_begin), d, tm);
    cp_async_commit();
    cp_async_wait_all();
    tm.sync();
    elem_copy_data<T>(vec(0), fac(0), pslot(0), d, n, stride, N, tm);
    if (e_begin + 1 < e_end) elem_copy_ptrs<T>(pslot(1), in, mats, entry(e_begin + 1), d, tm);
    cp_async_commit();

    for (long long ei = e_begin; ei < e_end; ++ei) {
        const int s = (int)((ei - e_begin) & 1);
        TO *o = out[entry(ei)];
        cp_async_wait_all();
        tm.sync();  // data of ei and pointers of ei+1 are in shared memory for the whole team
        if (ei + 1 < e_end) {
            elem_copy_data<T>(vec(s ^ 1), fac(s ^ 1), pslot(s ^ 1), d, n, stride, N, tm);
            if (ei + 2 < e_end) elem_copy_ptrs<T>(pslot(s), in, mats, entry(ei + 2), d, tm);
        }
        cp_async_commit();
        T *buf = vec(s);
        T y[EMAX];
        for (int i = d - 1; i >= 0; --i) {
            const T *M = fac(s) + i * P;
#pragma unroll
            for (int j = 0; j < EMAX; ++j) {
                const int q = tm.rank + j * tm.size;
                if (q < N) {
                    const int c = q / n, r = q - c * n;
                    const T *x = buf + c * n;
                    T sum = T(0);
#pragma unroll 8
                    for (int k = 0; k < n; ++k) sum = fma_t<T>(M[r + k * n], x[k], sum);
                    y[j] = sum;
                }
            }
            tm.sync();  // every read of this slot for this mode is done
            if (i > 0) {
#pragma unroll
                for (int j = 0; j < EMAX; ++j) {
                    const int q = tm.rank + j * tm.size;
                    if (q < N) {
                        const int c = q / n, r = q - c * n;
                        buf[c + r * F] = y[j];
                    }
                }
                tm.sync();
            }
        }
        if (o != cur) {
            if (cur != nullptr) flush(cur);
            cur = o;
#pragma unroll
            for (int j = 0; j < EMAX; ++j) acc[j] = y[j];
        } else {
#pragma unroll
            for (int j = 0; j < EMAX; ++j) acc[j] += y[j];
        }
    }
    if (cur != nullptr) flush(cur);
    cp_async_wait_all();
}

template <typename T, typename TO, int NN, int QMAX>
__global__ void __launch_bounds__(512, sizeof(T) == 4 ? 2 : 1) fwd_smem_kernel(const FwdArgs<T, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    const long long team_global = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    const long long e = team_global * a.entries_per_team;
    const long long e_end = min(e + (long long)a.entries_per_team, a.nb);
    if constexpr (FactorInSmem<T, NN>::value) {
        if (a.prefetch == 3) {  // ping-pong: three vector buffers, then two factor slots
            T *vb1 = buf + a.vec_pad, *vb2 = vb1 + a.vec_pad;
            T *fb0 = vb2 + a.vec_pad, *fb1 = fb0 + a.fac_pad;
            team_forward_pp<T, TO, NN, QMAX, false>(a.mats, a.in, a.out, a.d, a.stride, a.N, e, e_end, buf, vb1,
                                                     vb2, fb0, fb1, tm);
            return;
        }
    }
    if (a.prefetch) {
        T *buf2 = fac + a.fac_pad;
        T *fac2 = buf2 + a.vec_pad;
        team_forward<T, TO, NN, QMAX, false, true>(a.mats, a.in, a.out, nullptr, a.d, a.stride, a.N, e, e_end, buf,
                                                   fac, tm, buf2, fac2);
    } else {
        team_forward<T, TO, NN, QMAX, false>(a.mats, a.in, a.out, nullptr, a.d, a.stride, a.N, e, e_end, buf, fac,
                                             tm);
    }
}

// One entry per team, no run accumulator and no second staging slot: fewer
// registers and less shared memory, so more CTAs per SM.  The hardware block
// scheduler then overlaps one CTA's staging with other CTAs' compute.  Teams of
// at most 256 threads.
template <typename T, typename TO, int NN, int QMAX>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3) fwd_single_kernel(const FwdArgs<T, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    const long long e = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (e >= a.nb) return;
    const int F = a.N / NN;
    constexpr bool kSwz = VecSwizzle<T, NN>::on;
    stage_vector<T, kSwz>(buf, a.in[e], a.N, tm);
    stage_factors<T, NN>(fac, a.mats + e * a.d, a.d, a.stride, tm);
    tm.sync();
    T y[QMAX][NN];
    for (int i = a.d - 1; i >= 0; --i) {
        const T *M = fac + i * NN * NN;
        // small factors are read from shared memory per use (the compiler keeps them
        // in registers where it can); large ones a column at a time
        mode_team<T, NN, QMAX, kSwz, !FactorInSmem<T, NN>::value>(buf, M, M, F, tm, y);
        if (i > 0) {
            tm.sync();
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
    TO *o = a.out[e];
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
#pragma unroll
            for (int r = 0; r < NN; ++r) atomic_add<TO>(o + c + r * F, (TO)y[q][r]);
        }
    }
}

// The element mapping with n known at compile time: each thread owns up to EMAX
// output elements of every mode (consecutive lanes take consecutive rows of one
// fibre, which they read with the fibre's widest aligned loads as a broadcast), so
// the team's lanes stay busy whatever F is, while the index arithmetic and the
// k-loop are resolved at compile time.  Same k-ascending FMA chain per element as the
// fibre kernels (bitwise the same values).  FP64 only: there the pipe is charged per
// warp instruction whatever the number of active lanes.
template <typename T, typename TO, int NN, int EMAX>
__global__ void __launch_bounds__(256, 3) fwd_single_elem_kernel(const FwdArgs<T, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    const long long e = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (e >= a.nb) return;
    const int N = a.N, F = N / NN;
    constexpr int P = NN * NN;
    stage_vector(buf, a.in[e], N, tm);
    stage_factors<T, NN>(fac, a.mats + e * a.d, a.d, a.stride, tm);
    tm.sync();
    T y[EMAX];
    for (int i = a.d - 1; i >= 0; --i) {
        const T *M = fac + i * P;
#pragma unroll
        for (int j = 0; j < EMAX; ++j) {
            const int q = tm.rank + j * tm.size;  // row r = q % NN of fibre c = q / NN
            if (q < N) {
                const int c = q / NN, r = q - c * NN;
                T x[NN];
                load_fibre<T, NN>(buf + c * NN, x);
                T s = T(0);
#pragma unroll
                for (int k = 0; k < NN; ++k) s = fma_t<T>(M[r + k * NN], x[k], s);
                y[j] = s;
            }
        }
        if (i > 0) {
            tm.sync();
#pragma unroll
            for (int j = 0; j < EMAX; ++j) {
                const int q = tm.rank + j * tm.size;
                if (q < N) {
                    const int c = q / NN, r = q - c * NN;
                    buf[c + r * F] = y[j];
                }
            }
            tm.sync();
        }
    }
    TO *o = a.out[e];
#pragma unroll
    for (int j = 0; j < EMAX; ++j) {
        const int q = tm.rank + j * tm.size;
        if (q < N) {
            const int c = q / NN, r = q - c * NN;
            atomic_add<TO>(o + c + r * F, (TO)y[j]);
        }
    }
}

// ---- large vectors: global-memory sweep (compile-time n) -------------------
//
// For n^d beyond one SM's shared memory (the reference's large benchmark: n = 8,
// d = 6, N = 262144) the sweep streams through the caller's `input` and
// `workspace` vectors, which it overwrites as the reference does
// (kronmult_gpu/kronmult.cu:119-121).  One CTA per entry; every thread handles whole
// fibres (16-byte vector loads of a fibre, n outputs per fibre in registers,
// stores coalesced across the CTA); the factor of the current mode sits in shared
// memory; the last mode adds straight into the output with atomics, so there is no
// extra pass over the result.  One 512-thread CTA per entry, scheduled by the
// hardware (no persistent tail).  In FP64 the FP64 pipe stays the bound: the HBM
// traffic of 2N values per mode is an order of magnitude below its time.
template <typename T, typename TO, int NN>
__global__ void __launch_bounds__(512) fwd_global_kernel(const FwdArgs<T, TO> a)
{
    __shared__ T fac[NN * NN];
    const int N = a.N, F = N / NN, d = a.d;
    for (long long e = blockIdx.x; e < a.nb; e += gridDim.x) {
        T *src = const_cast<T *>(a.in[e]);
        T *dst = a.ws[e];
        TO *o = a.out[e];
        for (int i = d - 1; i >= 0; --i) {
            const T *A = a.mats[e * d + i];
            __syncthreads();  // previous mode finished with fac and with its src/dst
            for (int v = threadIdx.x; v < NN * NN; v += blockDim.x) {
                const int k = v / NN, r = v - k * NN;
                fac[v] = A[r + (size_t)k * a.stride];
            }
            __syncthreads();
            T m[NN * NN <= 16 ? NN * NN : 1];
            if constexpr (NN * NN <= 16) {
#pragma unroll
                for (int j = 0; j < NN * NN; ++j) m[j] = fac[j];
            }
            for (int c = threadIdx.x; c < F; c += blockDim.x) {
                T xv[NN];
                const T *x = src + (size_t)c * NN;
                if constexpr ((NN * sizeof(T)) % 16 == 0) {
#pragma unroll
                    for (int v = 0; v < (int)(NN * sizeof(T) / 16); ++v)
                        *reinterpret_cast<int4 *>(&xv[v * 16 / sizeof(T)]) = reinterpret_cast<const int4 *>(x)[v];
                } else {
#pragma unroll
                    for (int k = 0; k < NN; ++k) xv[k] = x[k];
                }
#pragma unroll
                for (int r = 0; r < NN; ++r) {
                    T s = T(0);
#pragma unroll
                    for (int k = 0; k < NN; ++k) {
                        const T mv = (NN * NN <= 16) ? m[(NN * NN <= 16) ? r + k * NN : 0] : fac[r + k * NN];
                        s = fma_t<T>(mv, xv[k], s);
                    }
                    if (i > 0) {
                        dst[c + (size_t)r * F] = s;
                    } else {
                        atomic_add<TO>(o + c + (size_t)r * F, (TO)s);
                    }
                }
            }
            T *t = src;
            src = dst;
            dst = t;
        }
    }
}

// ---- generic kernel (runtime n, any N) ------------------------------------
//
// One CTA per entry (grid-stride over entries), one thread per output element.
// Uses two shared-memory buffers when 2N values fit; otherwise it ping-pongs
// through the caller's `input` and `workspace` vectors in global memory, which it
// then clobbers, as the reference does (kronmult_gpu/kronmult.cu:119-121).
template <typename T, typename TO>
__global__ void __launch_bounds__(256) fwd_generic_kernel(const FwdArgs<T, TO> a, int use_smem)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = a.N, n = a.n, d = a.d;
    const int F = (n > 0) ? N / n : 0;
    T *fac = reinterpret_cast<T *>(smem_raw);  // n*n, transposed-free copy of the current factor
    T *s0 = fac + ((n * n + 1) & ~1);
    T *s1 = s0 + ((N + 1) & ~1);
    for (long long e = blockIdx.x; e < a.nb; e += gridDim.x) {
        const T *x = a.in[e];
        TO *o = a.out[e];
        T *src, *dst;
        if (use_smem) {
            for (int v = threadIdx.x; v < N; v += blockDim.x) s0[v] = x[v];
            src = s0;
            dst = s1;
        } else {
            src = const_cast<T *>(x);
            dst = a.ws[e];
        }
        __syncthreads();
        for (int i = d - 1; i >= 0; --i) {
            const T *A = a.mats[e * d + i];
            for (int v = threadIdx.x; v < n * n; v += blockDim.x) {
                const int k = v / n, r = v - k * n;
                fac[v] = A[r + (size_t)k * a.stride];
            }
            __syncthreads();
            for (int p = threadIdx.x; p < N; p += blockDim.x) {
                const int r = p / F, c = p - r * F;
                T s = T(0);
                for (int k = 0; k < n; ++k) s = fma_t<T>(fac[r + k * n], src[k + (size_t)c * n], s);
                dst[p] = s;
            }
            __syncthreads();
            T *t = src;
            src = dst;
            dst = t;
        }
        for (int p = threadIdx.x; p < N; p += blockDim.x) atomic_add<TO>(o + p, (TO)src[p]);
        __syncthreads();
    }
}

// kernel pointer lookup, defined once per (T, TO) instantiation unit
template <typename T, typename TO> using FwdSmemFn = void (*)(const FwdArgs<T, TO>);
template <typename T, typename TO> FwdSmemFn<T, TO> fwd_smem_lookup(int nn, int qmax);
template <typename T, typename TO> FwdSmemFn<T, TO> fwd_single_lookup(int nn, int qmax);
template <typename T, typename TO> FwdSmemFn<T, TO> fwd_single_elem_lookup(int nn, int emax);
template <typename T, typename TO> FwdSmemFn<T, TO> fwd_global_lookup(int nn);
template <typename T, typename TO> FwdSmemFn<T, TO> split_pass1_lookup(int nn, int qmax);
template <typename T, typename TO> FwdSmemFn<T, TO> split_pass2_lookup(int nn);
template <typename T, typename TO> void *fwd_generic_ptr();

}  // namespace kgb

// the element-mapped kernels of one n (lookup key n * 32 + EMAX)
#define KGB_ELEM_CASES(T, TO, NN)                                                                     \
    case NN * 32 + 1: return fwd_single_elem_kernel<T, TO, NN, 1>;                                    \
    case NN * 32 + 2: return fwd_single_elem_kernel<T, TO, NN, 2>;                                    \
    case NN * 32 + 4: return fwd_single_elem_kernel<T, TO, NN, 4>;                                    \
    case NN * 32 + 8: return fwd_single_elem_kernel<T, TO, NN, 8>;

// explicit instantiation of the forward kernels for one (T, TO) pair
#define KGB_FWD_INSTANTIATE(T, TO)                                                                     \
    namespace kgb {                                                                                    \
    template <> FwdSmemFn<T, TO> fwd_smem_lookup<T, TO>(int nn, int qmax)                             \
    {                                                                                                  \
        switch (nn * 16 + qmax) {                                                                      \
        case 2 * 16 + 1: return fwd_smem_kernel<T, TO, 2, 1>;                                          \
        case 2 * 16 + 2: return fwd_smem_kernel<T, TO, 2, 2>;                                          \
        case 2 * 16 + 4: return fwd_smem_kernel<T, TO, 2, 4>;                                          \
        case 2 * 16 + 8: return fwd_smem_kernel<T, TO, 2, 8>;                                          \
        case 3 * 16 + 1: return fwd_smem_kernel<T, TO, 3, 1>;                                          \
        case 3 * 16 + 2: return fwd_smem_kernel<T, TO, 3, 2>;                                          \
        case 3 * 16 + 4: return fwd_smem_kernel<T, TO, 3, 4>;                                          \
        case 3 * 16 + 8: return fwd_smem_kernel<T, TO, 3, 8>;                                          \
        case 4 * 16 + 1: return fwd_smem_kernel<T, TO, 4, 1>;                                          \
        case 4 * 16 + 2: return fwd_smem_kernel<T, TO, 4, 2>;                                          \
        case 4 * 16 + 4: return fwd_smem_kernel<T, TO, 4, 4>;                                          \
        case 4 * 16 + 8: return fwd_smem_kernel<T, TO, 4, 8>;                                          \
        case 5 * 16 + 1: return fwd_smem_kernel<T, TO, 5, 1>;                                          \
        case 5 * 16 + 2: return fwd_smem_kernel<T, TO, 5, 2>;                                          \
        case 5 * 16 + 4: return fwd_smem_kernel<T, TO, 5, 4>;                                          \
        case 6 * 16 + 1: return fwd_smem_kernel<T, TO, 6, 1>;                                          \
        case 6 * 16 + 2: return fwd_smem_kernel<T, TO, 6, 2>;                                          \
        case 6 * 16 + 4: return fwd_smem_kernel<T, TO, 6, 4>;                                          \
        case 7 * 16 + 1: return fwd_smem_kernel<T, TO, 7, 1>;                                          \
        case 7 * 16 + 2: return fwd_smem_kernel<T, TO, 7, 2>;                                          \
        case 7 * 16 + 4: return fwd_smem_kernel<T, TO, 7, 4>;                                          \
        case 8 * 16 + 1: return fwd_smem_kernel<T, TO, 8, 1>;                                          \
        case 8 * 16 + 2: return fwd_smem_kernel<T, TO, 8, 2>;                                          \
        case 8 * 16 + 4: return fwd_smem_kernel<T, TO, 8, 4>;                                          \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> FwdSmemFn<T, TO> fwd_single_lookup<T, TO>(int nn, int qmax)                           \
    {                                                                                                  \
        switch (nn * 16 + qmax) {                                                                      \
        case 2 * 16 + 1: return fwd_single_kernel<T, TO, 2, 1>;                                        \
        case 2 * 16 + 2: return fwd_single_kernel<T, TO, 2, 2>;                                        \
        case 2 * 16 + 4: return fwd_single_kernel<T, TO, 2, 4>;                                        \
        case 2 * 16 + 8: return fwd_single_kernel<T, TO, 2, 8>;                                        \
        case 3 * 16 + 1: return fwd_single_kernel<T, TO, 3, 1>;                                        \
        case 3 * 16 + 2: return fwd_single_kernel<T, TO, 3, 2>;                                        \
        case 3 * 16 + 4: return fwd_single_kernel<T, TO, 3, 4>;                                        \
        case 3 * 16 + 8: return fwd_single_kernel<T, TO, 3, 8>;                                        \
        case 4 * 16 + 1: return fwd_single_kernel<T, TO, 4, 1>;                                        \
        case 4 * 16 + 2: return fwd_single_kernel<T, TO, 4, 2>;                                        \
        case 4 * 16 + 4: return fwd_single_kernel<T, TO, 4, 4>;                                        \
        case 4 * 16 + 8: return fwd_single_kernel<T, TO, 4, 8>;                                        \
        case 5 * 16 + 1: return fwd_single_kernel<T, TO, 5, 1>;                                        \
        case 5 * 16 + 2: return fwd_single_kernel<T, TO, 5, 2>;                                        \
        case 5 * 16 + 4: return fwd_single_kernel<T, TO, 5, 4>;                                        \
        case 6 * 16 + 1: return fwd_single_kernel<T, TO, 6, 1>;                                        \
        case 6 * 16 + 2: return fwd_single_kernel<T, TO, 6, 2>;                                        \
        case 6 * 16 + 4: return fwd_single_kernel<T, TO, 6, 4>;                                        \
        case 7 * 16 + 1: return fwd_single_kernel<T, TO, 7, 1>;                                        \
        case 7 * 16 + 2: return fwd_single_kernel<T, TO, 7, 2>;                                        \
        case 7 * 16 + 4: return fwd_single_kernel<T, TO, 7, 4>;                                        \
        case 8 * 16 + 1: return fwd_single_kernel<T, TO, 8, 1>;                                        \
        case 8 * 16 + 2: return fwd_single_kernel<T, TO, 8, 2>;                                        \
        case 8 * 16 + 4: return fwd_single_kernel<T, TO, 8, 4>;                                        \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> FwdSmemFn<T, TO> fwd_single_elem_lookup<T, TO>(int nn, int emax)                       \
    {                                                                                                  \
        if constexpr (sizeof(T) == 8) {                                                                \
            switch (nn * 32 + emax) {                                                                  \
                KGB_ELEM_CASES(T, TO, 2)                                                              \
                KGB_ELEM_CASES(T, TO, 3)                                                              \
                KGB_ELEM_CASES(T, TO, 4)                                                              \
                KGB_ELEM_CASES(T, TO, 5)                                                              \
                KGB_ELEM_CASES(T, TO, 6)                                                              \
                KGB_ELEM_CASES(T, TO, 7)                                                              \
                KGB_ELEM_CASES(T, TO, 8)                                                              \
            default: return nullptr;                                                                   \
            }                                                                                          \
        } else {                                                                                       \
            return nullptr;                                                                            \
        }                                                                                              \
    }                                                                                                  \
    template <> FwdSmemFn<T, TO> fwd_global_lookup<T, TO>(int nn)                                     \
    {                                                                                                  \
        switch (nn) {                                                                                  \
        case 2: return fwd_global_kernel<T, TO, 2>;                                                    \
        case 3: return fwd_global_kernel<T, TO, 3>;                                                    \
        case 4: return fwd_global_kernel<T, TO, 4>;                                                    \
        case 5: return fwd_global_kernel<T, TO, 5>;                                                    \
        case 6: return fwd_global_kernel<T, TO, 6>;                                                    \
        case 7: return fwd_global_kernel<T, TO, 7>;                                                    \
        case 8: return fwd_global_kernel<T, TO, 8>;                                                    \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> void *fwd_generic_ptr<T, TO>() { return (void *)fwd_generic_kernel<T, TO>; }          \
    }
