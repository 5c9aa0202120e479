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
    long long nb;
    int d, stride, N, team_size, teams_per_cta, team_elems, vpad;
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

template <int NN, int QMAX> __global__ void __launch_bounds__(256, 3) df_single_kernel(const DfArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_emax[256 / 8 * 32];  // per team: vector scale + reduction space (<= 32 slots)
    const Team tm(a.team_size);
    constexpr int NN2 = NN * NN;
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
    const int width = tm.size < 32 ? tm.size : 32;
    for (int o = width / 2; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(tm.mask, m, o, width));
    if (tm.size > 32) {
        if ((tm.rank & 31) == 0) red[tm.rank >> 5] = m;
        tm.sync();
        m = 0;
        for (int w = 0; w < tm.size / 32; ++w) m = max(m, red[w]);
        tm.sync();
    }
    const int xe = m;
    const double *const *mats = a.mats + e * d;
    for (int i = tm.rank; i < d; i += tm.size) {
        int fm = 0;
        for (int k = 0; k < NN; ++k)
            for (int r = 0; r < NN; ++r) fm = max(fm, dexp(mats[i][r + (size_t)k * a.stride]));
        fexp[i] = fm;
    }
    tm.sync();
    // ---- split into hi/lo floats
    for (int v = tm.rank; v < N; v += tm.size) df_split(x[v], xe, xh[v], xl[v]);
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
                float bh[NN], bl[NN];
#pragma unroll
                for (int k = 0; k < NN; ++k) {
                    bh[k] = xh[k + c * NN];
                    bl[k] = xl[k + c * NN];
                }
#pragma unroll
                for (int r = 0; r < NN; ++r) {
                    // The error-free steps use explicitly rounded operations so that the
                    // compiler cannot fuse a product into a later addition.
                    // k = 0: the sum starts as the exact product
                    float ah = Mh[r], al = Ml[r];
                    float sh = __fmul_rn(ah, bh[0]);
                    float sl = fmaf(ah, bh[0], -sh);
                    sl = fmaf(ah, bl[0], sl);
                    sl = fmaf(al, bh[0], sl);
#pragma unroll
                    for (int k = 1; k < NN; ++k) {
                        ah = Mh[r + k * NN];
                        al = Ml[r + k * NN];
                        const float p = __fmul_rn(ah, bh[k]);  // two-product: p + ep = ah*bh exactly
                        float ep = fmaf(ah, bh[k], -p);
                        ep = fmaf(ah, bl[k], ep);              // cross terms
                        ep = fmaf(al, bh[k], ep);
                        const float t = __fadd_rn(sh, p);      // two-sum: t + err = sh + p exactly
                        const float bp = __fsub_rn(t, sh);
                        const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
                        sh = t;
                        sl = __fadd_rn(sl, __fadd_rn(err, ep));
                    }
                    const float h = __fadd_rn(sh, sl);  // renormalise: h + l = sh + sl
                    yl[q][r] = __fsub_rn(sl, __fsub_rn(h, sh));
                    yh[q][r] = h;
                }
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
                        xh[c + r * F] = yh[q][r];
                        xl[c + r * F] = yl[q][r];
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

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" int kronmult_batched_f64_emulated_async(int matrix_count, int matrix_size,
                                                   const double *const *matrix_list_batched, int matrix_stride,
                                                   const double *const *input_batched,
                                                   double *const *output_batched, int nb_batch, void *stream)
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
    // team: whole fibres per thread, at most 4 per thread, at most 256 threads
    int ts = 8;
    while (ts < 256 && ts * 2 < F) ts *= 2;
    while (ts < 256 && (F + ts - 1) / ts > 4) ts *= 2;
    const int q = (F + ts - 1) / ts;
    int qmax = 1;
    while (qmax < q) qmax *= 2;
    if (qmax > 4) return cudaErrorNotSupported;
    const DfFn fn = df_lookup(n, qmax);
    if (!fn) return cudaErrorNotSupported;
    DfArgs a{};
    a.mats = matrix_list_batched;
    a.in = input_batched;
    a.out = output_batched;
    a.nb = nb_batch;
    a.d = d;
    a.stride = matrix_stride;
    a.N = N;
    a.team_size = ts;
    a.vpad = round_up(N, 4);
    a.team_elems = 2 * a.vpad + round_up(2 * d * n * n + d, 4);
    int teams = 256 / ts;
    while (teams > 1 && (size_t)teams * a.team_elems * 4 > (size_t)di.max_smem_optin - 4096) teams /= 2;
    const size_t smem = (size_t)teams * a.team_elems * 4;
    if (smem > (size_t)di.max_smem_optin - 4096) return cudaErrorNotSupported;
    if (!ensure_smem_attr((const void *)fn, smem)) return cudaErrorInvalidValue;
    a.teams_per_cta = teams;
    const long long grid = (nb_batch + teams - 1) / teams;
    fn<<<(unsigned)grid, teams * ts, smem, (cudaStream_t)stream>>>(a);
    return (int)cudaGetLastError();
}
