// FP32 forward that applies two modes per shared-memory pass (n = 2 or 4).
//
// For FP32 the single-mode sweep is bound by shared-memory traffic (every mode
// reads and writes the whole vector once) rather than by HBM or the FMA pipe.
// Here a thread owns "bi-fibres": the n^2 contiguous values X[b + n*a + n^2*c2]
// that share every index except the two fastest ones (a, b).  It applies mode i
// to index b and mode i-1 to index a in registers, then writes the n^2 results
// to their twice-rotated positions
//     Z[c2 + F2*(r_b + n*r_a)],  F2 = N / n^2,
// which is exactly where two consecutive single-mode steps would put them
// (Y[c + r*F] twice), with the same k-ascending FMA chains.  An odd d starts with
// one single-mode step.  Shared-memory traffic and barriers are halved.
//
// Bank conflicts: for n = 4 a bi-fibre is 64 bytes per lane; its four 16-byte
// reads would hit the same banks every fourth lane.  The vector is therefore
// stored with 16-byte chunk ch at physical chunk ch ^ ((ch >> 3) & 7): eight
// consecutive bi-fibres then land in eight distinct bank groups, and the scalar
// writes of 32 consecutive positions stay a permutation of one 128-byte row.
#pragma once
#include "fwd_kernels.cuh"

namespace kgb {

template <int NN> struct PairSwizzle {
    // physical element index of logical element p (floats)
    static __device__ __forceinline__ int elem(int p)
    {
        if constexpr (NN == 4) {
            const int ch = p >> 2;
            return ((ch ^ ((ch >> 3) & 7)) << 2) | (p & 3);
        } else {
            return p;
        }
    }
    static __device__ __forceinline__ int chunk(int ch)
    {
        if constexpr (NN == 4) return ch ^ ((ch >> 3) & 7);
        return ch;
    }
};

// Pointers of one entry as seen by one thread: its input vector and the factor
// matrices of the (at most kPairFacSlots) factor elements this thread copies.
// They are loaded one entry ahead of the copy that uses them, so that the copy is
// not stalled behind dependent pointer-table loads.
constexpr int kPairFacSlots = 1;
struct PairPtrs {
    const float *src;
    const float *mat[kPairFacSlots];
};

template <int NN>
__device__ __forceinline__ void pair_load_ptrs(PairPtrs &p, const float *const *in, const float *const *mats,
                                               long long e, int d, const Team &tm)
{
    constexpr int NN2 = NN * NN;
    p.src = in[e];
#pragma unroll
    for (int s = 0; s < kPairFacSlots; ++s) {
        const int idx = tm.rank + s * tm.size;
        p.mat[s] = idx < d * NN2 ? mats[e * d + idx / NN2] : nullptr;
    }
}

// stage one entry (vector in the swizzled layout, factors plain) asynchronously
template <int NN>
__device__ __forceinline__ void pair_stage_async(float *dst, float *fac, const PairPtrs &p,
                                                 const float *const *mats_e, int N, int d, int stride, const Team &tm)
{
    if (((reinterpret_cast<uintptr_t>(p.src) & 15u) == 0) && ((N & 3) == 0)) {
        for (int v = tm.rank; v < N / 4; v += tm.size)
            cp_async<16>(dst + 4 * PairSwizzle<NN>::chunk(v), p.src + 4 * v);
    } else {
        for (int v = tm.rank; v < N; v += tm.size) cp_async<4>(dst + PairSwizzle<NN>::elem(v), p.src + v);
    }
    constexpr int NN2 = NN * NN;
#pragma unroll
    for (int s = 0; s < kPairFacSlots; ++s) {
        const int idx = tm.rank + s * tm.size;
        if (idx < d * NN2) {
            const int rem = idx % NN2, k = rem / NN, r = rem - k * NN;
            cp_async<4>(fac + idx, p.mat[s] + r + (size_t)k * stride);
        }
    }
    // elements beyond the prefetched slots (small teams only): direct pointer loads
    for (int idx = tm.rank + kPairFacSlots * tm.size; idx < d * NN2; idx += tm.size) {
        const int i = idx / NN2, rem = idx - i * NN2, k = rem / NN, r = rem - k * NN;
        cp_async<4>(fac + idx, mats_e[i] + r + (size_t)k * stride);
    }
    cp_async_commit();
}

// Team forward over entries [e_begin, e_end) with two staging slots; QP bi-fibres
// per thread.  Runs of equal output pointers are summed in registers (FP32) and
// added with atomics in the output type.
template <typename TO, int NN, int QP>
__device__ __forceinline__ void team_forward_pairs(const float *const *mats, const float *const *in, TO *const *out,
                                                   int d, int stride, int N, long long e_begin, long long e_end,
                                                   float *buf, float *fac, float *buf2, float *fac2, const Team &tm)
{
    using SW = PairSwizzle<NN>;
    constexpr int NN2 = NN * NN;
    constexpr int Q1 = QP * NN;  // fibres per thread in a single-mode step
    const int F = N / NN, F2 = N / NN2;
    float acc[QP][NN2];
    TO *cur = nullptr;

    PairPtrs nxt;
    if (e_begin < e_end) {
        pair_load_ptrs<NN>(nxt, in, mats, e_begin, d, tm);
        pair_stage_async<NN>(buf, fac, nxt, mats + e_begin * d, N, d, stride, tm);
        if (e_begin + 1 < e_end) pair_load_ptrs<NN>(nxt, in, mats, e_begin + 1, d, tm);
    }
    for (long long e = e_begin; e < e_end; ++e) {
        TO *o = out[e];
        cp_async_wait_all();
        tm.sync();
        if (e + 1 < e_end) {
            pair_stage_async<NN>(buf2, fac2, nxt, mats + (e + 1) * d, N, d, stride, tm);
            // pointers of entry e+2: in flight while entry e is computed
            if (e + 2 < e_end) pair_load_ptrs<NN>(nxt, in, mats, e + 2, d, tm);
        }

        int i = d - 1;
        if (d & 1) {
            // one single-mode step (mode d-1): fibres c = rank + q*size, q < Q1
            const float *M = fac + i * NN2;
            float y[Q1][NN];
#pragma unroll
            for (int q = 0; q < Q1; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
                    float xv[NN];
                    if constexpr (NN == 4) {
                        const float4 v = *reinterpret_cast<const float4 *>(buf + 4 * SW::chunk(c));
                        xv[0] = v.x;
                        xv[1] = v.y;
                        xv[2] = v.z;
                        xv[3] = v.w;
                    } else {
                        const float2 v = *reinterpret_cast<const float2 *>(buf + 2 * c);
                        xv[0] = v.x;
                        xv[1] = v.y;
                    }
#pragma unroll
                    for (int r = 0; r < NN; ++r) {
                        float s = 0.f;
#pragma unroll
                        for (int k = 0; k < NN; ++k) s = fmaf(M[r + k * NN], xv[k], s);
                        y[q][r] = s;
                    }
                }
            }
            tm.sync();
            // when F is a multiple of 256 the swizzle of c + r*F is the swizzle of c plus r*F
            const bool linear1 = NN != 4 || (F & 255) == 0;
#pragma unroll
            for (int q = 0; q < Q1; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
                    const int base = SW::elem(c);
#pragma unroll
                    for (int r = 0; r < NN; ++r) buf[linear1 ? base + r * F : SW::elem(c + r * F)] = y[q][r];
                }
            }
            tm.sync();
            --i;
        }
        float z[QP][NN2];
        for (; i >= 1; i -= 2) {
            const float *M1 = fac + i * NN2;        // acts on index b (fastest)
            const float *M0 = fac + (i - 1) * NN2;  // then on index a
#pragma unroll
            for (int q = 0; q < QP; ++q) {
                const int c2 = tm.rank + q * tm.size;
                if (c2 < F2) {
                    float x[NN][NN];
                    if constexpr (NN == 4) {
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            const float4 v = *reinterpret_cast<const float4 *>(buf + 4 * SW::chunk(4 * c2 + a));
                            x[a][0] = v.x;
                            x[a][1] = v.y;
                            x[a][2] = v.z;
                            x[a][3] = v.w;
                        }
                    } else {
                        const float4 v = *reinterpret_cast<const float4 *>(buf + 4 * c2);
                        x[0][0] = v.x;
                        x[0][1] = v.y;
                        x[1][0] = v.z;
                        x[1][1] = v.w;
                    }
                    // mode i on b, in place row by row
#pragma unroll
                    for (int a = 0; a < NN; ++a) {
                        float t[NN];
#pragma unroll
                        for (int rb = 0; rb < NN; ++rb) {
                            float s = 0.f;
#pragma unroll
                            for (int b = 0; b < NN; ++b) s = fmaf(M1[rb + b * NN], x[a][b], s);
                            t[rb] = s;
                        }
#pragma unroll
                        for (int rb = 0; rb < NN; ++rb) x[a][rb] = t[rb];
                    }
                    // mode i-1 on a, column by column
#pragma unroll
                    for (int rb = 0; rb < NN; ++rb) {
#pragma unroll
                        for (int ra = 0; ra < NN; ++ra) {
                            float s = 0.f;
#pragma unroll
                            for (int a = 0; a < NN; ++a) s = fmaf(M0[ra + a * NN], x[a][rb], s);
                            z[q][rb + NN * ra] = s;
                        }
                    }
                }
            }
            tm.sync();  // every read of buf (and fac) for this pass is done
            if (i > 1) {
                // when F2 is a multiple of 256 the swizzle of c2 + j*F2 is the swizzle of c2 plus j*F2
                const bool linear2 = NN != 4 || (F2 & 255) == 0;
#pragma unroll
                for (int q = 0; q < QP; ++q) {
                    const int c2 = tm.rank + q * tm.size;
                    if (c2 < F2) {
                        const int base = SW::elem(c2);
#pragma unroll
                        for (int j = 0; j < NN2; ++j) buf[linear2 ? base + F2 * j : SW::elem(c2 + F2 * j)] = z[q][j];
                    }
                }
                tm.sync();
            }
        }
        // z[q][rb + n*ra] is element c2 + F2*(rb + n*ra) of kron(A) . x
        if (o != cur) {
            if (cur != nullptr) {
#pragma unroll
                for (int q = 0; q < QP; ++q) {
                    const int c2 = tm.rank + q * tm.size;
                    if (c2 < F2) {
#pragma unroll
                        for (int j = 0; j < NN2; ++j) atomic_add<TO>(cur + c2 + F2 * j, (TO)acc[q][j]);
                    }
                }
            }
            cur = o;
#pragma unroll
            for (int q = 0; q < QP; ++q)
#pragma unroll
                for (int j = 0; j < NN2; ++j) acc[q][j] = z[q][j];
        } else {
#pragma unroll
            for (int q = 0; q < QP; ++q)
#pragma unroll
                for (int j = 0; j < NN2; ++j) acc[q][j] += z[q][j];
        }
        float *t = buf;
        buf = buf2;
        buf2 = t;
        t = fac;
        fac = fac2;
        fac2 = t;
    }
    if (cur != nullptr) {
#pragma unroll
        for (int q = 0; q < QP; ++q) {
            const int c2 = tm.rank + q * tm.size;
            if (c2 < F2) {
#pragma unroll
                for (int j = 0; j < NN2; ++j) atomic_add<TO>(cur + c2 + F2 * j, (TO)acc[q][j]);
            }
        }
    }
}

template <typename TO, int NN, int QP>
__global__ void __launch_bounds__(256, 3) fwd_pair_kernel(const FwdArgs<float, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    float *buf = reinterpret_cast<float *>(smem_raw) + (size_t)tm.id * a.team_elems;
    float *fac = buf + a.vec_pad;
    float *buf2 = fac + a.fac_pad;
    float *fac2 = buf2 + a.vec_pad;
    const long long team_global = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    const long long e = team_global * a.entries_per_team;
    const long long e_end = min(e + (long long)a.entries_per_team, a.nb);
    team_forward_pairs<TO, NN, QP>(a.mats, a.in, a.out, a.d, a.stride, a.N, e, e_end, buf, fac, buf2, fac2, tm);
}

template <typename TO> FwdSmemFn<float, TO> fwd_pair_lookup(int nn, int qp);

}  // namespace kgb

#define KGB_PAIR_INSTANTIATE(TO)                                                                       \
    namespace kgb {                                                                                    \
    template <> FwdSmemFn<float, TO> fwd_pair_lookup<TO>(int nn, int qp)                               \
    {                                                                                                  \
        switch (nn * 16 + qp) {                                                                        \
        case 2 * 16 + 1: return fwd_pair_kernel<TO, 2, 1>;                                             \
        case 2 * 16 + 2: return fwd_pair_kernel<TO, 2, 2>;                                             \
        case 4 * 16 + 1: return fwd_pair_kernel<TO, 4, 1>;                                             \
        case 4 * 16 + 2: return fwd_pair_kernel<TO, 4, 2>;                                             \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    }
