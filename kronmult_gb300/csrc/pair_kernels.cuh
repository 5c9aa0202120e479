// FP32 forward that applies two modes per shared-memory pass (n = 2, 4 and 8).
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
//
// n = 8 (team_forward_pairs8): a lane pair shares one 64-value bi-fibre X[a][b].
// Lane h holds rows a = 4h..4h+3 and applies mode i to them (index b); the pair then
// swaps halves with 16 shuffles so that lane h holds columns b = 4h..4h+3 of all 8
// rows, and applies mode i-1 to them (index a).  Each factor column is read as two
// 16-byte broadcast loads and feeds 32 FMAs; every output is still the k-ascending
// FMA chain from 0 of the reference.
#pragma once
#include "fwd_kernels.cuh"

namespace kgb {

template <int NN> struct PairSwizzle {
    // physical 16-byte chunk of logical chunk ch (n = 4): the XOR of bits 3..5 keeps every
    // aligned group of 8 chunks within itself (32 consecutive scalar positions stay one
    // 128-byte row) and puts 8 consecutive 64-byte bi-fibres on 8 slots.  (n = 8 uses
    // the padded layout of p8_phys instead.)
    static __device__ __forceinline__ int chunk(int ch)
    {
        if constexpr (NN == 4) return ch ^ ((ch >> 3) & 7);
        return ch;
    }
    // physical element index of logical element p (floats)
    static __device__ __forceinline__ int elem(int p)
    {
        if constexpr (NN == 4) {
            return (chunk(p >> 2) << 2) | (p & 3);
        } else {
            return p;
        }
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
                    if constexpr (NN == 4) {
                        // factor columns as 16-byte broadcast loads, FMAs in packed FP32
                        // pairs over the output index (each half the scalar k-ascending
                        // FMA chain from 0: the same bits)
                        const f2 zero2 = f2_pack(0.f, 0.f);
                        // mode i on b, in place row by row; column b of M1 as rows (0,1), (2,3)
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            f2 t0 = zero2, t1 = zero2;
#pragma unroll
                            for (int b = 0; b < 4; ++b) {
                                const float4 u = *reinterpret_cast<const float4 *>(M1 + 4 * b);
                                const f2 xb = f2_pack(x[a][b], x[a][b]);
                                t0 = f2_fma(f2_pack(u.x, u.y), xb, t0);
                                t1 = f2_fma(f2_pack(u.z, u.w), xb, t1);
                            }
                            f2_unpack(t0, x[a][0], x[a][1]);
                            f2_unpack(t1, x[a][2], x[a][3]);
                        }
                        // mode i-1 on a, column by column
#pragma unroll
                        for (int rb = 0; rb < 4; ++rb) {
                            f2 t0 = zero2, t1 = zero2;
#pragma unroll
                            for (int a = 0; a < 4; ++a) {
                                const float4 w = *reinterpret_cast<const float4 *>(M0 + 4 * a);
                                const f2 xa = f2_pack(x[a][rb], x[a][rb]);
                                t0 = f2_fma(f2_pack(w.x, w.y), xa, t0);
                                t1 = f2_fma(f2_pack(w.z, w.w), xa, t1);
                            }
                            f2_unpack(t0, z[q][rb], z[q][rb + 4]);
                            f2_unpack(t1, z[q][rb + 8], z[q][rb + 12]);
                        }
                    } else {
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

// ---- n = 8 --------------------------------------------------------------------

// Shared-memory layout of the n = 8 pair path: bi-fibre q (64 values) at 72 q + 16 (q/4),
// its two halves (rows 0..3 and 4..7, the halves of a lane pair) 36 floats apart.  The
// 16-byte loads of a warp's 8-lane phase (4 bi-fibres x 2 halves) start on 8 distinct
// bank slots; 32 consecutive positions stay within one 32-float half, and positions
// 4 bi-fibres apart (the two halves of a warp's stores for d = 4) land 304 floats
// apart, on the other 16 banks: the scalar stores are conflict-free.
__device__ __forceinline__ int p8_phys(int p)
{
    return (p >> 6) * 72 + (p >> 8) * 16 + ((p >> 5) & 1) * 36 + (p & 31);
}
__host__ __device__ constexpr int p8_elems(int N) { return N / 64 * 72 + N / 256 * 16; }

// factor elements a thread copies per entry through prefetched pointers (d*64 <= 4 x 64)
constexpr int kPair8FacSlots = 4;
struct Pair8Ptrs {
    const float *src;
    const float *mat[kPair8FacSlots];
};

__device__ __forceinline__ void pair8_load_ptrs(Pair8Ptrs &p, const float *const *in, const float *const *mats,
                                                long long e, int d, const Team &tm)
{
    p.src = in[e];
#pragma unroll
    for (int s = 0; s < kPair8FacSlots; ++s) {
        const int idx = tm.rank + s * tm.size;
        p.mat[s] = idx < d * 64 ? mats[e * d + (idx >> 6)] : nullptr;
    }
}

__device__ __forceinline__ void pair8_stage_async(float *dst, float *fac, const Pair8Ptrs &p,
                                                  const float *const *mats_e, int N, int d, int stride,
                                                  const Team &tm)
{
    if (((reinterpret_cast<uintptr_t>(p.src) & 15u) == 0) && ((N & 3) == 0)) {
        for (int v = tm.rank; v < N / 4; v += tm.size) cp_async<16>(dst + p8_phys(4 * v), p.src + 4 * v);
    } else {
        for (int v = tm.rank; v < N; v += tm.size) cp_async<4>(dst + p8_phys(v), p.src + v);
    }
#pragma unroll
    for (int s = 0; s < kPair8FacSlots; ++s) {
        const int idx = tm.rank + s * tm.size;
        if (idx < d * 64) {
            const int k = (idx >> 3) & 7, r = idx & 7;
            cp_async<4>(fac + idx, p.mat[s] + r + (size_t)k * stride);
        }
    }
    // elements beyond the prefetched slots (small teams only): direct pointer loads
    for (int idx = tm.rank + kPair8FacSlots * tm.size; idx < d * 64; idx += tm.size) {
        const int i = idx >> 6, k = (idx >> 3) & 7, r = idx & 7;
        cp_async<4>(fac + idx, mats_e[i] + r + (size_t)k * stride);
    }
    cp_async_commit();
}

// column k of a staged 8 x 8 factor (col-major, 16-byte aligned): two broadcast loads
__device__ __forceinline__ void factor_col8(const float *M, int k, float (&col)[8])
{
    const float4 u = *reinterpret_cast<const float4 *>(M + 8 * k);
    const float4 w = *reinterpret_cast<const float4 *>(M + 8 * k + 4);
    col[0] = u.x; col[1] = u.y; col[2] = u.z; col[3] = u.w;
    col[4] = w.x; col[5] = w.y; col[6] = w.z; col[7] = w.w;
}

// Team forward for n = 8 over entries [e_begin, e_end): a lane pair per bi-fibre
// (team = 2*F2 threads), two staging slots; runs of equal output pointers summed in
// registers (FP32) and added in the output type.  FMAs in packed FP32 pairs.
template <typename TO>
__device__ __forceinline__ void team_forward_pairs8(const float *const *mats, const float *const *in, TO *const *out,
                                                    int d, int stride, int N, long long e_begin, long long e_end,
                                                    float *buf, float *fac, float *buf2, float *fac2, const Team &tm)
{
    const int F = N / 8, F2 = N / 64;
    const int c2 = tm.rank >> 1;  // this lane pair's bi-fibre
    const int h = tm.rank & 1;    // rows 4h..4h+3, then columns 4h..4h+3
    const unsigned pair_mask = tm.size >= 32 ? 0xffffffffu : tm.mask;
    const f2 zero2 = f2_pack(0.f, 0.f);
    // destination of element c2 + F2*(4h + rr + 8 ra): for d = 4 (F2 = 64, c2 < 64) it is
    // p8_phys(c2) + 304 h + 72 rr + 608 ra (bi-fibre 4h + rr + 8 ra, group h + 2 ra)
    const bool lin = F2 == 64;
    const int dst0 = p8_phys(c2) + 304 * h;
    f2 acc[4][4];  // acc[rr][j] = elements (rr, ra = 2j), (rr, 2j+1)
    TO *cur = nullptr;

    Pair8Ptrs nxt;
    if (e_begin < e_end) {
        pair8_load_ptrs(nxt, in, mats, e_begin, d, tm);
        pair8_stage_async(buf, fac, nxt, mats + e_begin * d, N, d, stride, tm);
        if (e_begin + 1 < e_end) pair8_load_ptrs(nxt, in, mats, e_begin + 1, d, tm);
    }
    for (long long e = e_begin; e < e_end; ++e) {
        TO *o = out[e];
        cp_async_wait_all();
        tm.sync();
        if (e + 1 < e_end) {
            pair8_stage_async(buf2, fac2, nxt, mats + (e + 1) * d, N, d, stride, tm);
            if (e + 2 < e_end) pair8_load_ptrs(nxt, in, mats, e + 2, d, tm);
        }

        int i = d - 1;
        if (d & 1) {
            // one single-mode step (mode d-1) over the F fibres, at most 4 per thread
            const float *M = fac + i * 64;
            f2 y[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
                    const float *src = buf + p8_phys(8 * c);
                    const float4 u = *reinterpret_cast<const float4 *>(src);
                    const float4 w = *reinterpret_cast<const float4 *>(src + 4);
                    const float xv[8] = {u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w};
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const float4 m0 = *reinterpret_cast<const float4 *>(M + 8 * k);
                        const float4 m1 = *reinterpret_cast<const float4 *>(M + 8 * k + 4);
                        const f2 col[4] = {f2_pack(m0.x, m0.y), f2_pack(m0.z, m0.w), f2_pack(m1.x, m1.y),
                                           f2_pack(m1.z, m1.w)};
                        const f2 xk = f2_pack(xv[k], xv[k]);
#pragma unroll
                        for (int j = 0; j < 4; ++j) y[q][j] = f2_fma(col[j], xk, k == 0 ? zero2 : y[q][j]);
                    }
                }
            }
            tm.sync();
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float lo, hi;
                        f2_unpack(y[q][j], lo, hi);
                        buf[p8_phys(c + 2 * j * F)] = lo;
                        buf[p8_phys(c + (2 * j + 1) * F)] = hi;
                    }
                }
            }
            tm.sync();
            --i;
        }
        f2 z[4][4];  // z[rr][j]: elements c2 + F2*(4h + rr + 8 ra), ra = 2j, 2j+1
        for (; i >= 1; i -= 2) {
            const float *M1 = fac + i * 64;        // acts on index b (fastest)
            const float *M0 = fac + (i - 1) * 64;  // then on index a
            float x[4][8];                         // rows 4h + aa
            {
                const float *src = buf + p8_phys(64 * c2) + 36 * h;
#pragma unroll
                for (int aa = 0; aa < 4; ++aa) {
                    const float4 u = *reinterpret_cast<const float4 *>(src + 8 * aa);
                    const float4 w = *reinterpret_cast<const float4 *>(src + 8 * aa + 4);
                    x[aa][0] = u.x; x[aa][1] = u.y; x[aa][2] = u.z; x[aa][3] = u.w;
                    x[aa][4] = w.x; x[aa][5] = w.y; x[aa][6] = w.z; x[aa][7] = w.w;
                }
            }
            // mode i on b, for this lane's 4 rows
            {
                f2 t[4][4];
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const float4 m0 = *reinterpret_cast<const float4 *>(M1 + 8 * b);
                    const float4 m1 = *reinterpret_cast<const float4 *>(M1 + 8 * b + 4);
                    const f2 col[4] = {f2_pack(m0.x, m0.y), f2_pack(m0.z, m0.w), f2_pack(m1.x, m1.y),
                                       f2_pack(m1.z, m1.w)};
#pragma unroll
                    for (int aa = 0; aa < 4; ++aa) {
                        const f2 xb = f2_pack(x[aa][b], x[aa][b]);
#pragma unroll
                        for (int j = 0; j < 4; ++j) t[aa][j] = f2_fma(col[j], xb, b == 0 ? zero2 : t[aa][j]);
                    }
                }
#pragma unroll
                for (int aa = 0; aa < 4; ++aa)
#pragma unroll
                    for (int j = 0; j < 4; ++j) f2_unpack(t[aa][j], x[aa][2 * j], x[aa][2 * j + 1]);
            }
            // swap halves with the partner lane: keep columns 4h..4h+3 of the own rows,
            // send columns 4(1-h).. and receive the partner's rows at columns 4h..
            float lo[4][4], hi[4][4];  // rows 0..3 and 4..7 of this lane's 4 columns
#pragma unroll
            for (int aa = 0; aa < 4; ++aa) {
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const float own = h ? x[aa][4 + rr] : x[aa][rr];
                    const float send = h ? x[aa][rr] : x[aa][4 + rr];
                    const float recv = __shfl_xor_sync(pair_mask, send, 1);
                    lo[aa][rr] = h ? recv : own;
                    hi[aa][rr] = h ? own : recv;
                }
            }
            // mode i-1 on a, for this lane's 4 columns, a ascending
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const float4 m0 = *reinterpret_cast<const float4 *>(M0 + 8 * a);
                const float4 m1 = *reinterpret_cast<const float4 *>(M0 + 8 * a + 4);
                const f2 col[4] = {f2_pack(m0.x, m0.y), f2_pack(m0.z, m0.w), f2_pack(m1.x, m1.y),
                                   f2_pack(m1.z, m1.w)};
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const float xa = a < 4 ? lo[a & 3][rr] : hi[a & 3][rr];
                    const f2 x2 = f2_pack(xa, xa);
#pragma unroll
                    for (int j = 0; j < 4; ++j) z[rr][j] = f2_fma(col[j], x2, a == 0 ? zero2 : z[rr][j]);
                }
            }
            tm.sync();  // every read of buf (and fac) for this pass is done
            if (i > 1) {
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float v0, v1;
                        f2_unpack(z[rr][j], v0, v1);
                        const int r0 = rr + 8 * (2 * j), r1 = rr + 8 * (2 * j + 1);
                        if (lin) {
                            buf[dst0 + 72 * rr + 608 * (2 * j)] = v0;
                            buf[dst0 + 72 * rr + 608 * (2 * j + 1)] = v1;
                        } else {
                            buf[p8_phys(c2 + F2 * (4 * h + r0))] = v0;
                            buf[p8_phys(c2 + F2 * (4 * h + r1))] = v1;
                        }
                    }
                }
                tm.sync();
            }
        }
        if (o != cur) {
            if (cur != nullptr) {
#pragma unroll
                for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float v0, v1;
                        f2_unpack(acc[rr][j], v0, v1);
                        atomic_add<TO>(cur + c2 + F2 * (4 * h + rr + 8 * (2 * j)), (TO)v0);
                        atomic_add<TO>(cur + c2 + F2 * (4 * h + rr + 8 * (2 * j + 1)), (TO)v1);
                    }
            }
            cur = o;
#pragma unroll
            for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[rr][j] = z[rr][j];
        } else {
#pragma unroll
            for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[rr][j] = f2_add(acc[rr][j], z[rr][j]);
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
        for (int rr = 0; rr < 4; ++rr)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float v0, v1;
                f2_unpack(acc[rr][j], v0, v1);
                atomic_add<TO>(cur + c2 + F2 * (4 * h + rr + 8 * (2 * j)), (TO)v0);
                atomic_add<TO>(cur + c2 + F2 * (4 * h + rr + 8 * (2 * j + 1)), (TO)v1);
            }
    }
}

// One CTA of 128 threads: teams of 2*F2 threads (128 for d = 4, 16 for d = 3).
template <typename TO> __global__ void __launch_bounds__(128, 3) fwd_pair8_kernel(const FwdArgs<float, TO> a)
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
    team_forward_pairs8<TO>(a.mats, a.in, a.out, a.d, a.stride, a.N, e, e_end, buf, fac, buf2, fac2, tm);
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

// ---- n = 4, d = 6: three modes per pass ------------------------------------------
//
// For n = 4 a pass over bi-fibres does 4 FMAs per value per mode against one shared-
// memory read and write of every value, so two modes per pass leave the shared-memory
// traffic as large as the FMA work.  Here a lane pair owns a 64-value tri-fibre
// X[cc][a][b] (the three fastest indices, 4 each) and applies three modes per pass:
// lane h holds cc = 2h, 2h+1 (32 values), applies mode i to index b and mode i-1 to
// index a in registers, swaps with its partner half of the results (16 shuffles) so
// that it holds all four cc for rb = 2h, 2h+1, and applies mode i-2 to index cc.  The
// results go to their thrice-rotated positions
//     Z[c3 + 64 (rb + 4 ra + 16 rc)]      (N = 4096, 64 tri-fibres)
// where three single-mode steps would put them, each the same k-ascending FMA chain from
// 0 (bitwise the reference float kernel).  Two passes instead of three; the first
// writes its results into a middle buffer, so an entry needs two team barriers.
//
// Packed FP32 pairs (f2) hold the same element of two fibres, so that a factor value
// duplicated in both halves multiplies both fibres in one instruction and no value is
// duplicated in registers: the fibres (cl = 0, 1) for modes b and a, then (rb = 2h,
// 2h + 1) for mode cc.  Shared-memory layouts: tri-fibre c at 72 c, its half h at +36 h;
// there value (cl, a, b) at +16 cl + 4 a + b as the input lies (t4_in, staged in 16-byte
// copies) and at +8 a + 2 b + cl as the first pass writes it (t4_phys, read as pairs by
// the second); the factors of an entry duplicated,
// A_i(r, k) at words i*32 + 2 (r + 4 k) + {0, 1}.  Lane pairs are assigned tri-fibres
// (tri4_c3) so that the half-tri-fibre loads and the scattered stores of a pass are
// free of bank conflicts.  Lane h = 1 computes mode b's rows in the order r ^ 2, so
// that the rows each lane keeps and sends sit in the same registers on both lanes.
__host__ __device__ constexpr int t4_in(int p) { return 72 * (p >> 6) + 36 * ((p >> 5) & 1) + (p & 31); }
__host__ __device__ constexpr int t4_phys(int p)
{
    return 72 * (p >> 6) + 36 * ((p >> 5) & 1) + 8 * ((p >> 2) & 3) + 2 * (p & 3) + ((p >> 4) & 1);
}
constexpr int kTri4N = 4096;
constexpr int kTri4Elems = kTri4N / 64 * 72;  // padded vector
constexpr int kTri4Fac = 6 * 32;              // duplicated factors of one entry

// tri-fibre c3 = b' + 4 a' + 16 cl' + 32 g of team rank `rank` (h = rank & 1): b' from
// rank bits 1-2, the low bit of a' from bit 3, cl' from bit 4; the high bit of a' and g
// from the warp index.  A warp's 32 stores of one result then fall on 32 banks.
__device__ __forceinline__ int tri4_c3(int rank)
{
    const int w = rank >> 5;
    return ((rank >> 1) & 3) + 4 * (((rank >> 3) & 1) + 2 * (w & 1)) + 16 * ((rank >> 4) & 1) + 32 * (w >> 1);
}

__device__ __forceinline__ float f2_lo(f2 v)
{
    float lo, hi;
    f2_unpack(v, lo, hi);
    return lo;
}
__device__ __forceinline__ float f2_hi(f2 v)
{
    float lo, hi;
    f2_unpack(v, lo, hi);
    return hi;
}

template <typename TO>
__device__ __forceinline__ void flush_tri4(TO *dst, const f2 (&acc)[4][4], int c3, int h)
{
#pragma unroll
    for (int ra = 0; ra < 4; ++ra)
#pragma unroll
        for (int rc = 0; rc < 4; ++rc) {
            TO *o = dst + c3 + 64 * (2 * h + 4 * ra + 16 * rc);
            atomic_add<TO>(o, (TO)f2_lo(acc[ra][rc]));
            atomic_add<TO>(o + 64, (TO)f2_hi(acc[ra][rc]));
        }
}

template <typename TO>
__device__ __forceinline__ void team_forward_tri4(const float *const *mats, const float *const *in, TO *const *out,
                                                  int stride, long long e_begin, long long e_end, float *buf,
                                                  float *fac, float *buf2, float *fac2, float *mid, const Team &tm)
{
    const int c3 = tri4_c3(tm.rank);
    const int h = tm.rank & 1;
    const int src0 = 72 * c3 + 36 * h;             // + 8 a + 4 u: (cl, a, b = 2u, 2u + 1)
    const int dst0 = t4_phys(c3) + 144 * h;        // + 72 j + 288 ra + 1152 rc
    const int rowp = 4 * h;                        // word offset of row 2h in a duplicated column
    const f2 zero2 = f2_pack(0.f, 0.f);
    // -0 + w == w for every w (signed zeros and NaNs included): a run sum starts at -0
    const f2 nzero2 = f2_pack(-0.f, -0.f);
    f2 acc[4][4];  // acc[ra][rc] = run sums of elements (rc, ra, rb = 2h) and (rc, ra, 2h + 1)
#pragma unroll
    for (int ra = 0; ra < 4; ++ra)
#pragma unroll
        for (int rc = 0; rc < 4; ++rc) acc[ra][rc] = nzero2;
    TO *cur = nullptr;

    // the next entry's pointers, loaded one entry ahead: its input and (rank < 96) the
    // factor holding the rank-th of the entry's 96 factor values
    const float *nsrc = nullptr, *nmat = nullptr;
    TO *nout = nullptr;  // the output of the entry after the current one
    auto load_ptrs = [&](long long e) {
        nsrc = in[e];
        nout = out[e];
        nmat = tm.rank < 96 ? mats[e * 6 + (tm.rank >> 4)] : nullptr;
    };
    // the input goes in as it lies (t4_in), in 16-byte copies where aligned
    const int in16 = 72 * (tm.rank >> 4) + 36 * ((tm.rank >> 3) & 1) + 4 * (tm.rank & 7);  // t4_in(4 rank)
    const int in4 = 72 * (tm.rank >> 6) + 36 * ((tm.rank >> 5) & 1) + (tm.rank & 31);      // t4_in(rank)
    auto stage = [&](float *dst, float *fdst) {
        if ((reinterpret_cast<uintptr_t>(nsrc) & 15u) == 0) {
#pragma unroll
            for (int m = 0; m < 8; ++m) cp_async<16>(dst + in16 + 576 * m, nsrc + 4 * tm.rank + 512 * m);
        } else {
#pragma unroll 8
            for (int m = 0; m < 32; ++m) cp_async<4>(dst + in4 + 144 * m, nsrc + tm.rank + 128 * m);
        }
        if (nmat != nullptr) {  // A_i(r, k), rank = 16 i + 4 k + r, twice
            const float *g = nmat + (tm.rank & 3) + (size_t)((tm.rank >> 2) & 3) * stride;
            cp_async<4>(fdst + 2 * tm.rank, g);
            cp_async<4>(fdst + 2 * tm.rank + 1, g);
        }
        cp_async_commit();
    };
    TO *o = nullptr;  // the current entry's output
    if (e_begin < e_end) {
        load_ptrs(e_begin);
        stage(buf, fac);
        o = nout;
        if (e_begin + 1 < e_end) load_ptrs(e_begin + 1);
    }
    for (long long e = e_begin; e < e_end; ++e) {
        cp_async_wait_all();
        tm.sync();
        TO *const o_next = nout;
        if (e + 1 < e_end) {
            stage(buf2, fac2);
            if (e + 2 < e_end) load_ptrs(e + 2);
        }
        // a new output: write out the previous run's sums and start the next run
        if (o != cur) {
            if (cur != nullptr) {
                flush_tri4<TO>(cur, acc, c3, h);
#pragma unroll
                for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                    for (int rc = 0; rc < 4; ++rc) acc[ra][rc] = nzero2;
            }
            cur = o;
        }
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
            const float *M2 = fac + (5 - 3 * pass) * 32;  // mode on b
            const float *M1 = M2 - 32;                    // then on a
            const float *M0 = M2 - 64;                    // then on cc
            f2 X[4][4];                                   // X[a][b] = fibres (cl 0, cl 1)
            if (pass == 0) {  // the input layout: paired here
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(buf + src0 + 4 * a);
                    const float4 v1 = *reinterpret_cast<const float4 *>(buf + src0 + 16 + 4 * a);
                    X[a][0] = f2_pack(v0.x, v1.x);
                    X[a][1] = f2_pack(v0.y, v1.y);
                    X[a][2] = f2_pack(v0.z, v1.z);
                    X[a][3] = f2_pack(v0.w, v1.w);
                }
            } else {  // written paired by the first pass
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(mid + src0 + 8 * a + 4 * u);
                        X[a][2 * u] = v.x;
                        X[a][2 * u + 1] = v.y;
                    }
            }
            // mode on b; Y[a][r] holds row r ^ 2h
            f2 Y[4][4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int r = 0; r < 4; ++r) Y[a][r] = zero2;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const ulonglong2 m01 = *reinterpret_cast<const ulonglong2 *>(M2 + 8 * b + rowp);
                const ulonglong2 m23 = *reinterpret_cast<const ulonglong2 *>(M2 + 8 * b + (rowp ^ 4));
                const f2 m[4] = {m01.x, m01.y, m23.x, m23.y};
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int r = 0; r < 4; ++r) Y[a][r] = f2_fma(m[r], X[a][b], Y[a][r]);
            }
            // mode on a; Z[ra][r] holds rb = r ^ 2h
            f2 Z[4][4];
#pragma unroll
            for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                for (int r = 0; r < 4; ++r) Z[ra][r] = zero2;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const ulonglong2 m01 = *reinterpret_cast<const ulonglong2 *>(M1 + 8 * a);
                const ulonglong2 m23 = *reinterpret_cast<const ulonglong2 *>(M1 + 8 * a + 4);
                const f2 m[4] = {m01.x, m01.y, m23.x, m23.y};
#pragma unroll
                for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                    for (int r = 0; r < 4; ++r) Z[ra][r] = f2_fma(m[ra], Y[a][r], Z[ra][r]);
            }
            // keep Z[ra][j] (rb = 2h + j), send Z[ra][2 + j]; receive the partner's
            // cc = 2(1 - h) + cl at rb = 2h + j.  V[ra][cc] = fibres (rb 2h, rb 2h + 1)
            f2 V[4][4];
#pragma unroll
            for (int ra = 0; ra < 4; ++ra) {
                const float s00 = f2_lo(Z[ra][2]), s01 = f2_lo(Z[ra][3]);  // cl 0, j = 0, 1
                const float s10 = f2_hi(Z[ra][2]), s11 = f2_hi(Z[ra][3]);  // cl 1
                const f2 r0 = f2_pack(__shfl_xor_sync(0xffffffffu, s00, 1), __shfl_xor_sync(0xffffffffu, s01, 1));
                const f2 r1 = f2_pack(__shfl_xor_sync(0xffffffffu, s10, 1), __shfl_xor_sync(0xffffffffu, s11, 1));
                const f2 o0 = f2_pack(f2_lo(Z[ra][0]), f2_lo(Z[ra][1]));
                const f2 o1 = f2_pack(f2_hi(Z[ra][0]), f2_hi(Z[ra][1]));
                V[ra][0] = h ? r0 : o0;
                V[ra][1] = h ? r1 : o1;
                V[ra][2] = h ? o0 : r0;
                V[ra][3] = h ? o1 : r1;
            }
            // mode on cc, cc ascending
            f2 W[4][4];  // W[ra][rc]
#pragma unroll
            for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                for (int rc = 0; rc < 4; ++rc) W[ra][rc] = zero2;
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                const ulonglong2 m01 = *reinterpret_cast<const ulonglong2 *>(M0 + 8 * cc);
                const ulonglong2 m23 = *reinterpret_cast<const ulonglong2 *>(M0 + 8 * cc + 4);
                const f2 m[4] = {m01.x, m01.y, m23.x, m23.y};
#pragma unroll
                for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                    for (int rc = 0; rc < 4; ++rc) W[ra][rc] = f2_fma(m[rc], V[ra][cc], W[ra][rc]);
            }
            if (pass == 1) {  // into the run sums
#pragma unroll
                for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                    for (int rc = 0; rc < 4; ++rc) acc[ra][rc] = f2_add(acc[ra][rc], W[ra][rc]);
            } else {  // into the middle buffer (its last reads were the previous entry's)
#pragma unroll
                for (int ra = 0; ra < 4; ++ra)
#pragma unroll
                    for (int rc = 0; rc < 4; ++rc) {
                        mid[dst0 + 288 * ra + 1152 * rc] = f2_lo(W[ra][rc]);
                        mid[dst0 + 72 + 288 * ra + 1152 * rc] = f2_hi(W[ra][rc]);
                    }
                tm.sync();
            }
        }
        o = o_next;
        float *t = buf;
        buf = buf2;
        buf2 = t;
        t = fac;
        fac = fac2;
        fac2 = t;
    }
    if (cur != nullptr) flush_tri4<TO>(cur, acc, c3, h);
}

template <typename TO> __global__ void __launch_bounds__(128, 4) fwd_tri4_kernel(const FwdArgs<float, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(128);
    float *buf = reinterpret_cast<float *>(smem_raw);
    float *fac = buf + kTri4Elems;
    float *buf2 = fac + kTri4Fac;
    float *fac2 = buf2 + kTri4Elems;
    float *mid = fac2 + kTri4Fac;  // the first pass's results
    // CTA b runs entries [b nb / G, (b + 1) nb / G) of a grid of G
    const long long e = (long long)blockIdx.x * a.nb / gridDim.x;
    const long long e_end = (long long)(blockIdx.x + 1) * a.nb / gridDim.x;
    team_forward_tri4<TO>(a.mats, a.in, a.out, a.stride, e, e_end, buf, fac, buf2, fac2, mid, tm);
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
        case 8 * 16 + 1: return fwd_pair8_kernel<TO>;                                                  \
        case 4 * 16 + 3: return fwd_tri4_kernel<TO>; /* d = 6: three modes per pass */                 \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    }
