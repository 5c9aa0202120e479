// Double-float (FP32 pair) arithmetic for the FP64-accurate forward on the FP32 pipe,
// shared by the single-call kernels (df_kernels.cu) and the grouped persistent kernels
// (grouped_df.cu).
//
// Every value is an unevaluated sum hi + lo of two floats (48 significand bits).
// Products use the exact FMA two-product (p = a_h*b_h, e = fma(a_h, b_h, -p)) plus the
// two cross terms; sums use Knuth's two-sum (Dekker 1971, Knuth TAOCP vol. 2 4.2.2);
// each output is renormalised once.  Before splitting, an entry's vector is scaled by a
// power of two so that its largest magnitude is in [1, 2), and every factor likewise;
// the scales are undone exactly when the result is converted back.  Values more than
// 2^126 below the largest of their vector or factor are flushed to zero (their
// contribution is below the normwise error).
#pragma once
#include <cstdint>
#include "fwd_kernels.cuh"

namespace kgb {

// biased exponent field of a double (0 for zero/denormal, 2047 for inf/nan)
__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7FF); }

// x * 2^(1023 - emax) split into hi + lo floats (x's exponent field <= emax)
__device__ __forceinline__ void df_split(double x, int emax, float &hi, float &lo)
{
    const long long b = __double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF);
    const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
    if (E == 0x7FF || emax == 0x7FF) {  // inf / nan stay inf / nan
        hi = __int_as_float((int)(sign | 0x7F800000u | (((b & 0xFFFFFFFFFFFFFll) != 0) ? 0x400000u : 0u)));
        lo = 0.f;
        return;
    }
    const int u = E - emax;  // unbiased exponent after scaling, <= 0
    if (E == 0 || u < -126) {
        hi = __int_as_float((int)sign);
        lo = 0.f;
        return;
    }
    const unsigned long long mant = (unsigned long long)b & 0xFFFFFFFFFFFFFull;
    hi = __int_as_float((int)(sign | ((unsigned)(u + 127) << 23) | (unsigned)(mant >> 29)));
    const unsigned low = (unsigned)(mant & 0x1FFFFFFFu);  // the 29 bits below hi
    const int el = u - 52;                                 // weight of low's unit bit
    if (low == 0 || el < -126 - 29) {
        lo = 0.f;
        return;
    }
    // low * 2^el, rounded to 24 bits; exact power-of-two scaling in two steps keeps
    // the intermediate in the normal range
    float l = (float)low;
    l *= __int_as_float((unsigned)(el / 2 + 127) << 23);
    l *= __int_as_float((unsigned)(el - el / 2 + 127) << 23);
    lo = sign ? -l : l;
}

// float -> double times 2^s, exactly, with integer operations (zero/denormal -> 0)
__device__ __forceinline__ double f2d_scaled(float f, int s)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xFF;
    if (e == 0) return 0.0;
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    if (e == 0xFF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull |
                                                            ((unsigned long long)(b & 0x7FFFFF) << 29)));
    const long long E = (long long)e - 127 + 1023 + s;
    if (E <= 0) return 0.0;
    if (E >= 0x7FF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    return __longlong_as_double((long long)(sign | ((unsigned long long)E << 52) |
                                            ((unsigned long long)(b & 0x7FFFFF) << 29)));
}

// rows r, r + 1 of a column-major factor column: one 8-byte load when NN is even (r
// even, the factor arrays 8-byte aligned), two 4-byte loads otherwise
template <int NN> __device__ __forceinline__ f2 f2_rows(const float *p)
{
    if constexpr (NN % 2 == 0) {
        return *reinterpret_cast<const f2 *>(p);
    } else {
        return f2_pack(p[0], p[1]);
    }
}

// y = M . b for one fibre in double-float arithmetic: M (hi/lo) col-major NN x NN,
// b and y as hi/lo pairs.  Every output is the k-ascending sum of exact products,
// accumulated with two-sums and renormalised once.  Rows are computed two at a time
// in packed pairs (the same operations per row as the scalar form for an odd last row).
template <int NN>
__device__ __forceinline__ void df_fibre(const float *Mh, const float *Ml, const float (&bh)[NN],
                                         const float (&bl)[NN], float (&yh)[NN], float (&yl)[NN])
{
#pragma unroll
    for (int r = 0; r + 1 < NN; r += 2) {
        // k = 0: the sum starts as the exact product
        f2 ah = f2_rows<NN>(Mh + r), al = f2_rows<NN>(Ml + r);
        f2 b_h = f2_pack(bh[0], bh[0]), b_l = f2_pack(bl[0], bl[0]);
        f2 sh = f2_mul(ah, b_h);
        f2 sl = f2_fma(ah, b_h, f2_neg(sh));
        sl = f2_fma(ah, b_l, sl);
        sl = f2_fma(al, b_h, sl);
#pragma unroll
        for (int k = 1; k < NN; ++k) {
            ah = f2_rows<NN>(Mh + r + k * NN);
            al = f2_rows<NN>(Ml + r + k * NN);
            b_h = f2_pack(bh[k], bh[k]);
            b_l = f2_pack(bl[k], bl[k]);
            const f2 p = f2_mul(ah, b_h);  // two-product: p + ep = ah*bh exactly
            f2 ep = f2_fma(ah, b_h, f2_neg(p));
            ep = f2_fma(ah, b_l, ep);      // cross terms
            ep = f2_fma(al, b_h, ep);
            const f2 t = f2_add(sh, p);    // two-sum: t + err = sh + p exactly
            const f2 bp = f2_sub(t, sh);
            const f2 err = f2_add(f2_sub(sh, f2_sub(t, bp)), f2_sub(p, bp));
            sh = t;
            sl = f2_add(sl, f2_add(err, ep));
        }
        const f2 h = f2_add(sh, sl);  // renormalise: h + l = sh + sl
        const f2 l = f2_sub(sl, f2_sub(h, sh));
        f2_unpack(h, yh[r], yh[r + 1]);
        f2_unpack(l, yl[r], yl[r + 1]);
    }
    if constexpr (NN % 2 == 1) {
        constexpr int r = NN - 1;
        // The error-free steps use explicitly rounded operations so that the
        // compiler cannot fuse a product into a later addition.
        float ah = Mh[r], al = Ml[r];
        float sh = __fmul_rn(ah, bh[0]);
        float sl = fmaf(ah, bh[0], -sh);
        sl = fmaf(ah, bl[0], sl);
        sl = fmaf(al, bh[0], sl);
#pragma unroll
        for (int k = 1; k < NN; ++k) {
            ah = Mh[r + k * NN];
            al = Ml[r + k * NN];
            const float p = __fmul_rn(ah, bh[k]);
            float ep = fmaf(ah, bh[k], -p);
            ep = fmaf(ah, bl[k], ep);
            ep = fmaf(al, bh[k], ep);
            const float t = __fadd_rn(sh, p);
            const float bp = __fsub_rn(t, sh);
            const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
            sh = t;
            sl = __fadd_rn(sl, __fadd_rn(err, ep));
        }
        const float h = __fadd_rn(sh, sl);
        yl[r] = __fsub_rn(sl, __fsub_rn(h, sh));
        yh[r] = h;
    }
}

// largest exponent field over a team's values (team-wide; `red` >= 32 ints of shared memory)
__device__ __forceinline__ int team_max(int m, int *red, const Team &tm)
{
    const int width = tm.size < 32 ? tm.size : 32;
    for (int o = width / 2; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(tm.mask, m, o, width));
    if (tm.size > 32) {
        if ((tm.rank & 31) == 0) red[tm.rank >> 5] = m;
        tm.sync();
        m = 0;
        for (int w = 0; w < tm.size / 32; ++w) m = max(m, red[w]);
        tm.sync();
    }
    return m;
}

// team of whole fibres for F fibres: at most 4 per thread, at most 256 threads
// (0 when none fits); qmax = the power of two >= fibres per thread
inline int df_team(int F, int &qmax)
{
    int ts = 8;
    while (ts < 256 && ts * 2 < F) ts *= 2;
    while (ts < 256 && (F + ts - 1) / ts > 4) ts *= 2;
    const int q = (F + ts - 1) / ts;
    qmax = 1;
    while (qmax < q) qmax *= 2;
    return qmax > 4 ? 0 : ts;
}

// Shared-memory floats of one team's slice for one entry: the hi / lo vectors (vpad
// floats each, vpad = N rounded up to 4), the hi / lo factors and the d factor scales.
__host__ __device__ inline int df_slice_floats(int d, int n, int vpad)
{
    return 2 * vpad + (2 * d * n * n + d + 3) / 4 * 4;
}

// One entry's forward in double-float arithmetic by a team (the vector in xh / xl, the
// factors in mh / ml, their scales in fexp, `red` >= 32 ints for the team's
// reductions), whole fibres per thread, each mode in place through registers.
// emit(p, v) receives every output element p = c + r*F with its FP64 value.
template <int NN, int QMAX, typename Emit>
__device__ __forceinline__ void df_entry(const double *x, const double *const *mats, int d, int stride, int N,
                                         float *xh, float *xl, float *mh, float *ml, int *fexp, int *red,
                                         const Team &tm, Emit &&emit)
{
    constexpr int NN2 = NN * NN;
    constexpr bool kSwz = VecSwizzle<float, NN>::on;  // staged hi / lo vectors (n = 8: swizzled)
    const int F = N / NN;

    // ---- scales: largest exponent field of the vector and of every factor
    int m = 0;
    for (int v = tm.rank; v < N; v += tm.size) m = max(m, dexp(x[v]));
    const int xe = team_max(m, red, tm);
    for (int i = tm.rank; i < d; i += tm.size) {
        int fm = 0;
        for (int k = 0; k < NN; ++k)
            for (int r = 0; r < NN; ++r) fm = max(fm, dexp(mats[i][r + (size_t)k * stride]));
        fexp[i] = fm;
    }
    tm.sync();
    // ---- split into hi/lo floats
    for (int v = tm.rank; v < N; v += tm.size) {
        const int p = vec_pos<float, kSwz>(v);
        df_split(x[v], xe, xh[p], xl[p]);
    }
    for (int idx = tm.rank; idx < d * NN2; idx += tm.size) {
        const int i = idx / NN2, rem = idx - i * NN2, k = rem / NN, r = rem - k * NN;
        df_split(mats[i][r + (size_t)k * stride], fexp[i], mh[idx], ml[idx]);
    }
    int scale = xe - 1023;  // result = value * 2^scale
    for (int i = 0; i < d; ++i) scale += fexp[i] - 1023;
    tm.sync();

    float yh[QMAX][NN], yl[QMAX][NN];
    for (int i = d - 1; i >= 0; --i) {
        const float *Mh = mh + i * NN2, *Ml = ml + i * NN2;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int c = tm.rank + q * tm.size;
            if (c < F) {
                // whole-fibre vector loads (16-byte for n = 4, 8; the swizzled layout
                // for n = 8): consecutive lanes read consecutive fibres without bank
                // conflicts
                float bh[NN], bl[NN];
                load_fibre_v<float, NN, kSwz>(xh, c, bh);
                load_fibre_v<float, NN, kSwz>(xl, c, bl);
                df_fibre<NN>(Mh, Ml, bh, bl, yh[q], yl[q]);
            }
        }
        tm.sync();  // every read of this entry's shared memory for the mode is done
        if (i > 0) {
#pragma unroll
            for (int q = 0; q < QMAX; ++q) {
                const int c = tm.rank + q * tm.size;
                if (c < F) {
#pragma unroll
                    for (int r = 0; r < NN; ++r) {
                        const int p = vec_pos<float, kSwz>(c + r * F);
                        xh[p] = yh[q][r];
                        xl[p] = yl[q][r];
                    }
                }
            }
            tm.sync();
        }
    }
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
#pragma unroll
            for (int r = 0; r < NN; ++r) emit(c + r * F, f2d_scaled(yh[q][r], scale) + f2d_scaled(yl[q][r], scale));
        }
    }
}

}  // namespace kgb
