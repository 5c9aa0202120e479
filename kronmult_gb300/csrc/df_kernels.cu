// FP64-accurate forward emulated with double-float (FP32 pair) arithmetic.
//
// GB300's FP64 pipe delivers ~1.25 TFLOP/s against ~73 TFLOP/s of FP32, so every
// FP64 configuration of this path is bound by the FP64 pipe.  This kernel keeps
// FP64 inputs, factors and outputs but computes each mode product in
// "double-float" arithmetic: every value is an unevaluated sum hi + lo of two
// floats (48 significand bits).  Products use the exact FMA two-product
// (p = a_h*b_h, e = fma(a_h, b_h, -p)) plus the two cross terms; sums use Knuth's
// two-sum (Dekker 1971, Knuth TAOCP vol. 2 4.2.2); each output is renormalised once.
// The relative error per mode is a few units of 2^-47, far inside the 1e-13
// relative-L2 contract of the FP64 path.
//
// Range: before splitting, the entry's vector is scaled by a power of two so that
// its largest magnitude is in [1, 2), and every factor likewise; the scales are
// undone exactly when the result is converted back.  Values more than 2^126 below
// the largest of their vector or factor are flushed to zero (their contribution is
// below the normwise error).  The split and the conversions back use integer
// operations only, so the FP64 pipe does one addition per output element.
//
// Layout and mapping follow fwd_single_kernel: one team per entry, whole fibres per
// thread, each mode in place through registers, one FP64 atomic per output element.
#include <cstdint>
#include "fwd_launch.cuh"

namespace kgb {
namespace {

struct DfArgs {
    const double *const *mats;
    const double *const *in;
    double *const *out;
    double *const *ws;  // workspaces (two-pass path only)
    long long nb;
    int d, stride, N, team_size, teams_per_cta, team_elems, vpad;
    // two-pass path (vectors beyond shared memory): N = R x C, C = n^d1
    int d1, C, R, L, ept;
};

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

template <int NN, int QMAX> __global__ void __launch_bounds__(256, 3) df_single_kernel(const DfArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_emax[256 / 8 * 32];  // per team: vector scale + reduction space (<= 32 slots)
    const Team tm(a.team_size);
    constexpr int NN2 = NN * NN;
    constexpr bool kSwz = VecSwizzle<float, NN>::on;  // staged hi / lo vectors (n = 8: swizzled)
    float *xh = reinterpret_cast<float *>(smem_raw) + (size_t)tm.id * a.team_elems;
    float *xl = xh + a.vpad;
    float *mh = xl + a.vpad;                 // d * NN2
    float *ml = mh + a.d * NN2;              // d * NN2
    int *fexp = reinterpret_cast<int *>(ml + a.d * NN2);  // d factor scales
    int *red = s_emax + tm.id * 32;
    const long long e = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (e >= a.nb) return;
    const int N = a.N, F = N / NN, d = a.d;
    const double *x = a.in[e];

    // ---- scales: largest exponent field of the vector and of every factor
    int m = 0;
    for (int v = tm.rank; v < N; v += tm.size) m = max(m, dexp(x[v]));
    const int xe = team_max(m, red, tm);
    const double *const *mats = a.mats + e * d;
    for (int i = tm.rank; i < d; i += tm.size) {
        int fm = 0;
        for (int k = 0; k < NN; ++k)
            for (int r = 0; r < NN; ++r) fm = max(fm, dexp(mats[i][r + (size_t)k * a.stride]));
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
        df_split(mats[i][r + (size_t)k * a.stride], fexp[i], mh[idx], ml[idx]);
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
        tm.sync();
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
    double *o = a.out[e];
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
#pragma unroll
            for (int r = 0; r < NN; ++r)
                atomicAdd(o + c + r * F, f2d_scaled(yh[q][r], scale) + f2d_scaled(yl[q][r], scale));
        }
    }
}

// ---- vectors beyond shared memory: two passes through the workspace ----------
//
// N = R x C with C = n^d1 (the d1 fastest tensor indices), as in the FP32 two-pass
// sweep: the first d1 modes of the backward sweep act within contiguous chunks of C
// values, the last d - d1 within the R values sharing a fast position (stride C).
// Pass 1 sweeps every chunk in double-float arithmetic, scaled by the chunk's own
// largest exponent, and stores the FP64 result to the entry's workspace; pass 2
// sweeps tiles of L fast positions x R rows, scaled by the tile's largest exponent,
// and adds into the output.  The input is only read.

// Pass 1: one team per (entry, chunk); layout and mapping of df_single_kernel.
template <int NN, int QMAX> __global__ void __launch_bounds__(256, 3) df_pass1_kernel(const DfArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_emax[256 / 8 * 32];
    const Team tm(a.team_size);
    constexpr int NN2 = NN * NN;
    constexpr bool kSwz = VecSwizzle<float, NN>::on;
    const int C = a.C, F = C / NN, d1 = a.d1, d2 = a.d - d1;
    float *xh = reinterpret_cast<float *>(smem_raw) + (size_t)tm.id * a.team_elems;
    float *xl = xh + a.vpad;
    float *mh = xl + a.vpad;                 // d1 * NN2
    float *ml = mh + d1 * NN2;               // d1 * NN2
    int *fexp = reinterpret_cast<int *>(ml + d1 * NN2);
    int *red = s_emax + tm.id * 32;
    const long long w = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (w >= a.nb * (long long)a.R) return;
    const long long e = w / a.R;
    const size_t off = (size_t)(w - e * a.R) * (size_t)C;
    const double *x = a.in[e] + off;
    int m = 0;
    for (int v = tm.rank; v < C; v += tm.size) m = max(m, dexp(x[v]));
    const int xe = team_max(m, red, tm);
    const double *const *mats = a.mats + e * a.d + d2;  // the last d1 factors
    for (int i = tm.rank; i < d1; i += tm.size) {
        int fm = 0;
        for (int k = 0; k < NN; ++k)
            for (int r = 0; r < NN; ++r) fm = max(fm, dexp(mats[i][r + (size_t)k * a.stride]));
        fexp[i] = fm;
    }
    tm.sync();
    for (int v = tm.rank; v < C; v += tm.size) {
        const int p = vec_pos<float, kSwz>(v);
        df_split(x[v], xe, xh[p], xl[p]);
    }
    for (int idx = tm.rank; idx < d1 * NN2; idx += tm.size) {
        const int i = idx / NN2, rem = idx - i * NN2, k = rem / NN, r = rem - k * NN;
        df_split(mats[i][r + (size_t)k * a.stride], fexp[i], mh[idx], ml[idx]);
    }
    int scale = xe - 1023;
    for (int i = 0; i < d1; ++i) scale += fexp[i] - 1023;
    tm.sync();
    float yh[QMAX][NN], yl[QMAX][NN];
    for (int i = d1 - 1; i >= 0; --i) {
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
        tm.sync();
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
    double *dst = a.ws[e] + off;
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
#pragma unroll
            for (int r = 0; r < NN; ++r) dst[c + r * F] = f2d_scaled(yh[q][r], scale) + f2d_scaled(yl[q][r], scale);
        }
    }
}

// copy one entry's workspace tile (R rows of L values from column l0) and its first
// d2 factors (FP64, fr[i*NN2 + r + k*NN] = A_i(r, k)) into shared memory (cp.async)
template <int NN>
__device__ __forceinline__ void df_tile_async(double *raw, double *fr, const double *src, const double *const *mats,
                                              int R, int L, int C, int lw, int d2, int stride)
{
    for (int idx = threadIdx.x; idx < R * L; idx += blockDim.x) {
        const int h = idx / L, l = idx - h * L;
        if (l < lw) {
            cp_async<8>(raw + idx, src + (size_t)h * C + l);
        } else {
            raw[idx] = 0.0;
        }
    }
    constexpr int NN2 = NN * NN;
    for (int idx = threadIdx.x; idx < d2 * NN2; idx += blockDim.x) {
        const int i = idx / NN2, rem = idx - i * NN2, k = rem / NN, r = rem - k * NN;
        cp_async<8>(fr + idx, mats[i] + r + (size_t)k * stride);
    }
    cp_async_commit();
}

// largest exponent field over the CTA (256 threads; `red` >= 8 ints)
__device__ __forceinline__ int block_max(int m, int *red)
{
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = max(m, red[w]);
    return m;
}

// Pass 2: one CTA per (tile of L fast positions, range of entries); thread (fibre c,
// column l) as in the FP32 pass 2.  The next entry's tile and factors are copied while
// the current one is computed; runs of equal outputs are summed in an FP64 tile and
// flushed with atomics.
template <int NN> __global__ void __launch_bounds__(256, 2) df_pass2_kernel(const DfArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_red[8 + 8 * 8];
    constexpr int NN2 = NN * NN;
    const int R = a.R, L = a.L, C = a.C, d2 = a.d - a.d1, F = R / NN, RL = R * L;
    const int tiles = (C + L - 1) / L;
    double *acc = reinterpret_cast<double *>(smem_raw);  // R x L run sums
    double *raw0 = acc + RL;                               // two copy slots: tile, then factors
    double *raw1 = raw0 + RL + d2 * NN2;
    float *Sh = reinterpret_cast<float *>(raw1 + RL + d2 * NN2);
    float *Sl = Sh + RL;
    float *Dh = Sl + RL;
    float *Dl = Dh + RL;
    float *fh = Dl + RL;
    float *fl = fh + d2 * NN2;
    int *fexp = s_red + 8;  // d2 <= 8 factor scales (and their per-warp partials)
    const int l0 = (int)(blockIdx.x % tiles) * L;
    const int lw = min(L, C - l0);
    const long long e_begin = (long long)(blockIdx.x / tiles) * a.ept;
    const long long e_end = min(e_begin + (long long)a.ept, a.nb);
    double *cur = nullptr;
    auto flush = [&](double *dst) {
        for (int t = threadIdx.x; t < F * L; t += blockDim.x) {
            const int c = t / L, l = t - c * L;
            if (l < lw) {
#pragma unroll
                for (int r = 0; r < NN; ++r) atomicAdd(dst + (size_t)(c + r * F) * C + l0 + l, acc[(c + r * F) * L + l]);
            }
        }
    };
    if (e_begin < e_end)
        df_tile_async<NN>(raw0, raw0 + RL, a.ws[e_begin] + l0, a.mats + e_begin * a.d, R, L, C, lw, d2, a.stride);
    for (long long e = e_begin; e < e_end; ++e) {
        double *o = a.out[e];
        double *raw = ((e - e_begin) & 1) ? raw1 : raw0;
        const double *fr = raw + RL;
        cp_async_wait_all();
        __syncthreads();  // tile and factors of e complete; entry e-1 done with the other slot
        if (e + 1 < e_end)
            df_tile_async<NN>(((e - e_begin) & 1) ? raw0 : raw1, (((e - e_begin) & 1) ? raw0 : raw1) + RL,
                              a.ws[e + 1] + l0, a.mats + (e + 1) * a.d, R, L, C, lw, d2, a.stride);
        // scales: the tile's largest exponent, and each factor's
        int m = 0;
        for (int idx = threadIdx.x; idx < RL; idx += blockDim.x) m = max(m, dexp(raw[idx]));
        const int te = block_max(m, s_red);
        if (threadIdx.x < 32 * d2 && threadIdx.x < blockDim.x) {
            const int i = threadIdx.x >> 5, lane = threadIdx.x & 31;
            int fm = 0;
            for (int v = lane; v < NN2; v += 32) fm = max(fm, dexp(fr[i * NN2 + v]));
            for (int o2 = 16; o2 > 0; o2 >>= 1) fm = max(fm, __shfl_xor_sync(0xffffffffu, fm, o2));
            if (lane == 0) fexp[i] = fm;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < RL; idx += blockDim.x) df_split(raw[idx], te, Sh[idx], Sl[idx]);
        for (int idx = threadIdx.x; idx < d2 * NN2; idx += blockDim.x) df_split(fr[idx], fexp[idx / NN2], fh[idx], fl[idx]);
        int scale = te - 1023;
        for (int i = 0; i < d2; ++i) scale += fexp[i] - 1023;
        const bool fresh = o != cur;
        if (fresh && cur != nullptr) flush(cur);
        cur = o;
        __syncthreads();
        float *Xh = Sh, *Xl = Sl, *Yh = Dh, *Yl = Dl;
        for (int i = d2 - 1; i >= 0; --i) {
            const float *Mh = fh + i * NN2, *Ml = fl + i * NN2;
            for (int t = threadIdx.x; t < F * L; t += blockDim.x) {
                const int c = t / L, l = t - c * L;
                float bh[NN], bl[NN], yh[NN], yl[NN];
#pragma unroll
                for (int k = 0; k < NN; ++k) {
                    bh[k] = Xh[(k + c * NN) * L + l];
                    bl[k] = Xl[(k + c * NN) * L + l];
                }
                df_fibre<NN>(Mh, Ml, bh, bl, yh, yl);
                if (i > 0) {
#pragma unroll
                    for (int r = 0; r < NN; ++r) {
                        Yh[(c + r * F) * L + l] = yh[r];
                        Yl[(c + r * F) * L + l] = yl[r];
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < NN; ++r) {
                        double &sacc = acc[(c + r * F) * L + l];
                        const double v = f2d_scaled(yh[r], scale) + f2d_scaled(yl[r], scale);
                        sacc = fresh ? v : sacc + v;
                    }
                }
            }
            if (i > 0) {
                __syncthreads();
                float *t = Xh;
                Xh = Yh;
                Yh = t;
                t = Xl;
                Xl = Yl;
                Yl = t;
            }
        }
    }
    if (cur != nullptr) flush(cur);
    cp_async_wait_all();
}

using DfFn = void (*)(const DfArgs);

DfFn df_lookup(int nn, int qmax)
{
#define KGB_DF(NN, Q) \
    case NN * 16 + Q: return df_single_kernel<NN, Q>;
    switch (nn * 16 + qmax) {
        KGB_DF(2, 1) KGB_DF(2, 2) KGB_DF(2, 4)
        KGB_DF(3, 1) KGB_DF(3, 2) KGB_DF(3, 4)
        KGB_DF(4, 1) KGB_DF(4, 2) KGB_DF(4, 4)
        KGB_DF(5, 1) KGB_DF(5, 2) KGB_DF(5, 4)
        KGB_DF(6, 1) KGB_DF(6, 2) KGB_DF(6, 4)
        KGB_DF(7, 1) KGB_DF(7, 2) KGB_DF(7, 4)
        KGB_DF(8, 1) KGB_DF(8, 2) KGB_DF(8, 4)
    default: return nullptr;
    }
#undef KGB_DF
}

DfFn df_pass1_lookup(int nn, int qmax)
{
#define KGB_DF(NN, Q) \
    case NN * 16 + Q: return df_pass1_kernel<NN, Q>;
    switch (nn * 16 + qmax) {
        KGB_DF(2, 1) KGB_DF(2, 2) KGB_DF(2, 4)
        KGB_DF(3, 1) KGB_DF(3, 2) KGB_DF(3, 4)
        KGB_DF(4, 1) KGB_DF(4, 2) KGB_DF(4, 4)
        KGB_DF(5, 1) KGB_DF(5, 2) KGB_DF(5, 4)
        KGB_DF(6, 1) KGB_DF(6, 2) KGB_DF(6, 4)
        KGB_DF(7, 1) KGB_DF(7, 2) KGB_DF(7, 4)
        KGB_DF(8, 1) KGB_DF(8, 2) KGB_DF(8, 4)
    default: return nullptr;
    }
#undef KGB_DF
}

DfFn df_pass2_lookup(int nn)
{
    switch (nn) {
    case 2: return df_pass2_kernel<2>;
    case 3: return df_pass2_kernel<3>;
    case 4: return df_pass2_kernel<4>;
    case 5: return df_pass2_kernel<5>;
    case 6: return df_pass2_kernel<6>;
    case 7: return df_pass2_kernel<7>;
    case 8: return df_pass2_kernel<8>;
    default: return nullptr;
    }
}

// team of whole fibres for F fibres: at most 4 per thread, at most 256 threads
// (0 when none fits); qmax = the power of two >= fibres per thread
int df_team(int F, int &qmax)
{
    int ts = 8;
    while (ts < 256 && ts * 2 < F) ts *= 2;
    while (ts < 256 && (F + ts - 1) / ts > 4) ts *= 2;
    const int q = (F + ts - 1) / ts;
    qmax = 1;
    while (qmax < q) qmax *= 2;
    return qmax > 4 ? 0 : ts;
}

// two passes through the workspace for vectors beyond one team's shared memory
int df_two_pass(DfArgs a, int n, const DeviceInfo &di, cudaStream_t st)
{
    const int d = a.d;
    constexpr int kFloatAlign = 4;
    for (int d1 = d - 1; d1 >= 1; --d1) {
        const int d2 = d - d1;
        if (d2 > 8) return cudaErrorNotSupported;
        const long long C = pow_ll(n, d1), R = pow_ll(n, d2);
        if (R > 4096) return cudaErrorNotSupported;
        int qmax = 0;
        const int ts = df_team((int)(C / n), qmax);
        if (!ts) continue;
        const DfFn f1 = df_pass1_lookup(n, qmax), f2 = df_pass2_lookup(n);
        if (!f1 || !f2) return cudaErrorNotSupported;
        const int vpad = round_up((int)C, kFloatAlign);
        const int team_elems = 2 * vpad + round_up(2 * d1 * n * n + d1, kFloatAlign);
        int teams = 256 / ts;
        while (teams > 1 && (size_t)teams * team_elems * 4 > (size_t)di.max_smem_optin - 8192) teams /= 2;
        const size_t smem1 = (size_t)teams * team_elems * 4;
        if (smem1 > (size_t)di.max_smem_optin - 8192) continue;
        // pass-2 tile: rows of at least 128 bytes and 256 (fibre, position) tasks where
        // it fits in half the SM; narrower (32 bytes at least) otherwise
        const int F2 = (int)(R / n);
        auto smem2_of = [&](long long L) {
            const long long RL = R * L;
            return (size_t)(RL * 8 + 2 * (RL + d2 * n * n) * 8 + 4 * RL * 4 + 2 * d2 * n * n * 4);
        };
        int L = 16;
        while ((long long)L * F2 < 256 && L < 256) L *= 2;
        while (L > 4 && smem2_of(L) > (size_t)di.max_smem_optin / 2) L /= 2;
        const size_t smem2 = smem2_of(L);
        if (smem2 > (size_t)di.max_smem_optin) return cudaErrorNotSupported;
        const long long tiles = (C + L - 1) / L;
        long long ept = a.nb * tiles / (16LL * di.sms);
        if (ept > 64) ept = 64;
        if (ept < 1) ept = 1;
        const long long grid1 = (a.nb * R + teams - 1) / teams, grid2 = (a.nb + ept - 1) / ept * tiles;
        if (grid1 > INT_MAX || grid2 > INT_MAX) return cudaErrorInvalidValue;
        if (!ensure_smem_attr((const void *)f1, smem1) || !ensure_smem_attr((const void *)f2, smem2))
            return cudaErrorInvalidValue;
        a.team_size = ts;
        a.teams_per_cta = teams;
        a.team_elems = team_elems;
        a.vpad = vpad;
        a.d1 = d1;
        a.C = (int)C;
        a.R = (int)R;
        a.L = L;
        a.ept = (int)ept;
        f1<<<(unsigned)grid1, teams * ts, smem1, st>>>(a);
        f2<<<(unsigned)grid2, 256, smem2, st>>>(a);
        return (int)cudaGetLastError();
    }
    return cudaErrorNotSupported;
}

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" int kronmult_batched_f64_emulated_async(int matrix_count, int matrix_size,
                                                   const double *const *matrix_list_batched, int matrix_stride,
                                                   const double *const *input_batched,
                                                   double *const *output_batched, double *const *workspace_batched,
                                                   int nb_batch, void *stream)
{
    const int d = matrix_count, n = matrix_size;
    if (d < 0 || n < 0 || nb_batch < 0 || matrix_stride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    const long long Nl = pow_ll(n, d);
    if (Nl > (long long)INT_MAX) return cudaErrorInvalidValue;
    if (nb_batch == 0 || n == 0) return cudaSuccess;
    if (!matrix_list_batched || !input_batched || !output_batched) return cudaErrorInvalidValue;
    if (n < 2 || n > 8 || d < 1) return cudaErrorNotSupported;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);
    const int N = (int)Nl, F = N / n;
    DfArgs a{};
    a.mats = matrix_list_batched;
    a.in = input_batched;
    a.out = output_batched;
    a.ws = workspace_batched;
    a.nb = nb_batch;
    a.d = d;
    a.stride = matrix_stride;
    a.N = N;
    // one team per entry when the vector fits one team's shared memory
    int qmax = 0;
    const int ts = df_team(F, qmax);
    const DfFn fn = ts ? df_lookup(n, qmax) : nullptr;
    if (fn) {
        a.team_size = ts;
        a.vpad = round_up(N, 4);
        a.team_elems = 2 * a.vpad + round_up(2 * d * n * n + d, 4);
        int teams = 256 / ts;
        while (teams > 1 && (size_t)teams * a.team_elems * 4 > (size_t)di.max_smem_optin - 4096) teams /= 2;
        const size_t smem = (size_t)teams * a.team_elems * 4;
        if (smem <= (size_t)di.max_smem_optin - 4096) {
            if (!ensure_smem_attr((const void *)fn, smem)) return cudaErrorInvalidValue;
            a.teams_per_cta = teams;
            const long long grid = (nb_batch + teams - 1) / teams;
            fn<<<(unsigned)grid, teams * ts, smem, (cudaStream_t)stream>>>(a);
            return (int)cudaGetLastError();
        }
    }
    // larger vectors: two passes through the workspace
    if (!workspace_batched) return cudaErrorNotSupported;
    return df_two_pass(a, n, di, (cudaStream_t)stream);
}
