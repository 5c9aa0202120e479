// FP64 forward on the FP64 tensor path (mma.sync m8n8k4 .f64), for factor sizes
// whose mode product is a dense GEMM wide enough to fill the 8 x 8 MMA tile.
//
// A mode product Y[c + r*F] = sum_k A(r,k) X[k + c*n] (the Algorithm-993 step of
// kronmult_gpu/kronmult.cu:139-197 and kronmult_omp/kronmult.hpp:77-104) is, per tile
// of 8 fibres c, the product D (8 fibres x 8 rows r) = Xtile (8 x K) * A^T (K x 8), with
// K = n padded to a multiple of 4 and run as K/4 chained m8n8k4 MMAs.  On GB300 one
// m8n8k4 MMA computes every element of D as the k-ascending FMA chain
// fma(a3,b3, fma(a2,b2, fma(a1,b1, fma(a0,b0, c)))) -- bitwise, measured on random
// operands of mixed magnitude against that chain on the host (no other summation order
// matched) -- so chaining the K/4 MMAs from C = 0 gives exactly the chain the CUDA-core
// kernels and the reference compute, k = 0 .. n-1.  Padded k slots multiply 0 by 0 and
// add +0, which leaves every non-zero partial sum unchanged.
//
// Rate: on GB300 the FP64 tensor path and the FP64 FMA pipe are one resource -- with
// independent accumulators m8n8k4 runs about 1.08x the FMA work rate of DFMA, and warps
// issuing both take the sum of their times.  So the tensor path pays off where the 8 x 8
// tile is full and the FMA-pipe kernel is weak: n = 16, which the FMA pipe covers only
// with the generic run-time-n kernel (the tensor path: 1.8-2.1x faster than it).  For
// n = 6..8 the FMA-pipe kernels are faster (n = 8: by about 10 %), and for n = 9..15 the
// generic kernel beats a tensor path whose tile is 42-88 % busy (measured 1.2-3x); the
// tensor path stays selectable for n = 6..8 (kronmult_tuning.fp64_path = 2).
//
// Fragment layout (PTX ISA, mma m8n8k4 .f64): lane = 4g + s holds A(row g, col s),
// B(row s, col g) and D(row g, cols 2s and 2s+1).
#pragma once
#include "fwd_kernels.cuh"

namespace kgb {

template <int NN> struct DmmaShape {
    static constexpr int KC = (NN + 3) / 4;  // chained MMAs over k
    static constexpr int NB = (NN + 7) / 8;  // column blocks of 8 rows r
};

// D += A * B for one 8 x 8 x 4 FP64 tile (the accumulator in place)
__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b)
{
    asm("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
        : "+d"(d0), "+d"(d1)
        : "d"(a), "d"(b));
}

// This lane's B fragments of factor M (M[r + k*NN] = A(r,k)): B(k, r) = A(r, k), zero
// outside n x n.
template <int NN>
__device__ __forceinline__ void dmma_factor_frags(const double *M, double (&b)[DmmaShape<NN>::KC][DmmaShape<NN>::NB])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
#pragma unroll
    for (int kc = 0; kc < DmmaShape<NN>::KC; ++kc) {
#pragma unroll
        for (int nb = 0; nb < DmmaShape<NN>::NB; ++nb) {
            const int k = kc * 4 + s, r = nb * 8 + g;
            b[kc][nb] = (k < NN && r < NN) ? M[r + k * NN] : 0.0;
        }
    }
}

// The same from a factor in global memory (column-major, leading dimension `stride`).
template <int NN>
__device__ __forceinline__ void dmma_factor_frags_global(const double *A, int stride,
                                                         double (&b)[DmmaShape<NN>::KC][DmmaShape<NN>::NB])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
#pragma unroll
    for (int kc = 0; kc < DmmaShape<NN>::KC; ++kc) {
#pragma unroll
        for (int nb = 0; nb < DmmaShape<NN>::NB; ++nb) {
            const int k = kc * 4 + s, r = nb * 8 + g;
            b[kc][nb] = (k < NN && r < NN) ? A[r + (size_t)k * stride] : 0.0;
        }
    }
}

// One mode product of the vector in `buf` (X[k + c*NN], F fibres) for this warp's
// tiles t = w + q*W (q < QT, 8 fibres each) into D (registers).  Tiles at or beyond F
// are skipped (warp-uniform); rows beyond F read zeros.  FULL: every tile exists and
// is full (F == 8*W*QT), no checks.
template <int NN, int QT, bool FULL>
__device__ __forceinline__ void dmma_mode(const double *buf, const double (&b)[DmmaShape<NN>::KC][DmmaShape<NN>::NB],
                                          int F, int w, int W, double (&D)[QT][DmmaShape<NN>::NB][2])
{
    constexpr int KC = DmmaShape<NN>::KC, NB = DmmaShape<NN>::NB;
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
#pragma unroll
    for (int q = 0; q < QT; ++q)
#pragma unroll
        for (int nb = 0; nb < NB; ++nb) D[q][nb][0] = D[q][nb][1] = 0.0;
#pragma unroll
    for (int q = 0; q < QT; ++q) {
        const int t = w + q * W;
        if (FULL || t * 8 < F) {
            const int c = t * 8 + g;
            double av[KC];
#pragma unroll
            for (int kc = 0; kc < KC; ++kc) {
                const int k = kc * 4 + s;
                av[kc] = ((FULL || c < F) && (NN % 4 == 0 || k < NN)) ? buf[k + c * NN] : 0.0;
            }
#pragma unroll
            for (int kc = 0; kc < KC; ++kc)
#pragma unroll
                for (int nb = 0; nb < NB; ++nb) dmma_8x8x4(D[q][nb][0], D[q][nb][1], av[kc], b[kc][nb]);
        }
    }
}

// Writes D back as the next mode's vector, Y[c + r*F] (in place: the caller has
// synchronised the team after every read of the mode), or adds it into the output.
template <int NN, int QT, bool FULL, bool RED, typename TP>
__device__ __forceinline__ void dmma_emit(TP *dst, int F, int w, int W, const double (&D)[QT][DmmaShape<NN>::NB][2])
{
    constexpr int NB = DmmaShape<NN>::NB;
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
#pragma unroll
    for (int q = 0; q < QT; ++q) {
        const int t = w + q * W;
        const int c = t * 8 + g;
        if (FULL || c < F) {
#pragma unroll
            for (int nb = 0; nb < NB; ++nb)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int r = nb * 8 + 2 * s + j;
                    if (NN % 8 == 0 || r < NN) {
                        if constexpr (RED)
                            atomic_add<double>(dst + c + (size_t)r * F, D[q][nb][j]);
                        else
                            dst[c + (size_t)r * F] = D[q][nb][j];
                    }
                }
        }
    }
}

// One entry per team of W = team_size/32 warps; the vector and the d factors staged in
// shared memory, each mode's D held in registers until the team has read the whole
// vector, then written back in place; the last mode adds into the output with FP64
// atomics.  Same semantics as fwd_single_kernel, bitwise the same values.
template <int NN, int QT, bool FULL>
__global__ void __launch_bounds__(256) fwd_dmma_kernel(const FwdArgs<double, double> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int KC = DmmaShape<NN>::KC, NB = DmmaShape<NN>::NB;
    const Team tm(a.team_size);
    double *buf = reinterpret_cast<double *>(smem_raw) + (size_t)tm.id * a.team_elems;
    double *fac = buf + a.vec_pad;
    const long long e = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    if (e >= a.nb) return;
    const int F = a.N / NN, w = tm.rank >> 5, W = tm.size >> 5;
    stage_vector(buf, a.in[e], a.N, tm);
    stage_factors<double, NN>(fac, a.mats + e * a.d, a.d, a.stride, tm);
    tm.sync();
    double D[QT][NB][2];
    for (int i = a.d - 1; i >= 0; --i) {
        double b[KC][NB];
        dmma_factor_frags<NN>(fac + i * NN * NN, b);
        dmma_mode<NN, QT, FULL>(buf, b, F, w, W, D);
        if (i > 0) {
            tm.sync();
            dmma_emit<NN, QT, FULL, false>(buf, F, w, W, D);
            tm.sync();
        }
    }
    dmma_emit<NN, QT, FULL, true>(a.out[e], F, w, W, D);
}

// Vectors beyond shared memory (the reference's large benchmark shape n = 8, d = 6,
// N = 262144): the sweep streams through the caller's input and workspace vectors,
// which it overwrites as the reference does (kronmult_gpu/kronmult.cu:119-121).  One
// 512-thread CTA per entry (grid-stride); each warp takes groups of G tiles, loads their
// A fragments from global memory (the 8 fibres of a tile are 8*NN contiguous values),
// runs the chained MMAs and stores D to the workspace, or adds it into the output in
// the last mode.
template <int NN>
__global__ void __launch_bounds__(512) fwd_dmma_global_kernel(const FwdArgs<double, double> a)
{
    constexpr int KC = DmmaShape<NN>::KC, NB = DmmaShape<NN>::NB, G = 4;
    const int N = a.N, F = N / NN, d = a.d;
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
    const int w = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int tiles = (F + 7) / 8;
    for (long long e = blockIdx.x; e < a.nb; e += gridDim.x) {
        double *src = const_cast<double *>(a.in[e]);
        double *dst = a.ws[e];
        double *o = a.out[e];
        for (int i = d - 1; i >= 0; --i) {
            double b[KC][NB];
            dmma_factor_frags_global<NN>(a.mats[e * d + i], a.stride, b);
            __syncthreads();  // the previous mode's stores into src are visible
            for (int t0 = w * G; t0 < tiles; t0 += W * G) {
                double av[G][KC];
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    const int c = (t0 + q) * 8 + g;
#pragma unroll
                    for (int kc = 0; kc < KC; ++kc) {
                        const int k = kc * 4 + s;
                        av[q][kc] = (t0 + q < tiles && c < F && (NN % 4 == 0 || k < NN))
                                        ? __ldcg(src + k + (size_t)c * NN)
                                        : 0.0;
                    }
                }
                double D[G][NB][2];
#pragma unroll
                for (int q = 0; q < G; ++q)
#pragma unroll
                    for (int nb = 0; nb < NB; ++nb) D[q][nb][0] = D[q][nb][1] = 0.0;
#pragma unroll
                for (int kc = 0; kc < KC; ++kc)
#pragma unroll
                    for (int q = 0; q < G; ++q)
#pragma unroll
                        for (int nb = 0; nb < NB; ++nb) dmma_8x8x4(D[q][nb][0], D[q][nb][1], av[q][kc], b[kc][nb]);
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    const int c = (t0 + q) * 8 + g;
                    if (t0 + q < tiles && c < F) {
#pragma unroll
                        for (int nb = 0; nb < NB; ++nb)
#pragma unroll
                            for (int j = 0; j < 2; ++j) {
                                const int r = nb * 8 + 2 * s + j;
                                if (NN % 8 == 0 || r < NN) {
                                    if (i > 0)
                                        __stcg(dst + c + (size_t)r * F, D[q][nb][j]);
                                    else
                                        atomic_add<double>(o + c + (size_t)r * F, D[q][nb][j]);
                                }
                            }
                    }
                }
            }
            double *tmp = src;
            src = dst;
            dst = tmp;
        }
        __syncthreads();  // every thread is done with this entry's buffers
    }
}

using DmmaFn = void (*)(const FwdArgs<double, double>);
// fwd_dmma_kernel for (n, tiles per warp, full tiles); null where not instantiated
DmmaFn fwd_dmma_lookup(int nn, int qt, bool full);
DmmaFn fwd_dmma_global_lookup(int nn);
// n with a tensor-path instantiation
inline bool dmma_has_n(int nn) { return (nn >= 6 && nn <= 8) || nn == 16; }

}  // namespace kgb
