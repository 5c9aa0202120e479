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
#include "df_common.cuh"
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

template <int NN, int QMAX> __global__ void __launch_bounds__(256, 3) df_single_kernel(const DfArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_emax[256 / 8 * 32];  // per team: reduction space (<= 32 slots)
    const Team tm(a.team_size);
    constexpr int NN2 = NN * NN;
    float *xh = reinterpret_cast<float *>(smem_raw) + (size_t)tm.id * a.team_elems;
    float *xl = xh + a.vpad;
    float *mh = xl + a.vpad;                 // d * NN2
    float *ml = mh + a.d * NN2;              // d * NN2
    int *fexp = reinterpret_cast<int *>(ml + a.d * NN2);  // d factor scales
    const long long e = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (e >= a.nb) return;
    double *o = a.out[e];
    df_entry<NN, QMAX>(a.in[e], a.mats + e * a.d, a.d, a.stride, a.N, xh, xl, mh, ml, fexp, s_emax + tm.id * 32, tm,
                       [&](int p, double v) { atomic_add<double>(o + p, v); });
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
        size_t smem = (size_t)teams * a.team_elems * 4;
        if (smem <= (size_t)di.max_smem_optin - 4096) {
            if (!ensure_smem_attr((const void *)fn, smem)) return cudaErrorInvalidValue;
            long long grid = (nb_batch + teams - 1) / teams;
            // one wave or less: every SM holds the same number of CTAs (as the native planner)
            if (grid > di.sms) {
                const int occ = occupancy((const void *)fn, teams * ts, smem);
                if (grid <= (long long)occ * di.sms) {
                    const long long k = (grid + di.sms - 1) / di.sms;
                    const long long t2 = (nb_batch + k * di.sms - 1) / (k * di.sms);
                    if (t2 >= 1 && t2 < teams) {
                        teams = (int)t2;
                        smem = (size_t)teams * a.team_elems * 4;
                        grid = (nb_batch + teams - 1) / teams;
                    }
                }
            }
            a.teams_per_cta = teams;
            fn<<<(unsigned)grid, teams * ts, smem, (cudaStream_t)stream>>>(a);
            return (int)cudaGetLastError();
        }
    }
    // larger vectors: two passes through the workspace
    if (!workspace_batched) return cudaErrorNotSupported;
    return df_two_pass(a, n, di, (cudaStream_t)stream);
}
