// Diagnostic: measured FP64 fused-multiply-add rate of the current GPU.
//
// Every FP64 configuration of kronmult is bound by the FP64 pipe rather than by
// HBM (arithmetic intensity 1.5-5 flop/byte against a ridge near 0.2 flop/byte
// on GB300), so the roofline the benchmark reports for them is this measured rate.
#include <cuda_runtime.h>
#include "kronmult_gb300.h"

namespace {

__global__ void dfma_rate_kernel(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1234.5678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int kronmult_diag_fp64_fma_gflops(double *gflops)
{
    if (!gflops) return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return rc;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if ((rc = cudaMalloc(&out, sizeof(double))) != cudaSuccess) return rc;
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 4, threads = 256, iters = 1000;
    dfma_rate_kernel<<<blocks, threads, 0, st>>>(out, 16, 1.0000001, 1e-9);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, st);
        dfma_rate_kernel<<<blocks, threads, 0, st>>>(out, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    rc = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(out);
    if (rc != cudaSuccess) return rc;
    const double flops = 2.0 * 64.0 * iters * (double)blocks * threads;
    *gflops = flops / (best * 1e-3) / 1e9;
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Diagnostics behind the choice of FP64 arithmetic (no reference counterpart).
//
// kronmult_diag_fp64_mma_gflops: FP64 tensor-core (DMMA) throughput, from warps that
// issue independent mma.sync m8n8k4 f64 instructions out of registers.
// kronmult_diag_int8_mma_tops: INT8 tensor-core throughput, mma.sync m16n8k32 s8 -> s32.
// kronmult_diag_ozaki_elementwise_ms: the per-element work that an FP64 emulation by
// integer slices on tensor cores (the Ozaki scheme: error-free splitting of each
// operand into fixed-point 8-bit slices, integer products accumulated exactly, the
// slice levels recombined into FP64 -- Ozaki, Ogita and Oishi, Numer. Algorithms 2012)
// has to do outside the tensor cores for every element of every mode product: scale
// to fixed point, split into `slices` digits, and recombine `slices` levels of integer
// sums into FP64.  The kernel does exactly that work per element (one FP64 read and
// one FP64 write, everything else in registers) and no tensor-core work, so its time
// is a lower bound for the scheme on that many element-mode-products.
namespace {

__global__ void dmma_rate_kernel(double *out, int iters)
{
    const double a = 1.0 + 1e-9 * threadIdx.x, b = 1.0 - 1e-9 * threadIdx.x;
    double c[8][2];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[j][0]), "+d"(c[j][1])
                         : "d"(a), "d"(b));
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1];
    if (s == 1234.5678) out[0] = s;  // keeps the accumulators live
}

__global__ void imma_rate_kernel(int *out, int iters)
{
    const unsigned a = 0x01010101u * (threadIdx.x & 7), b = 0x02020202u;
    int c[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            asm volatile(
                "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
                "{%0, %1, %2, %3};"
                : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
                : "r"(a), "r"(a), "r"(a), "r"(a), "r"(b), "r"(b));
    }
    int s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
    if (s == 123456789) out[0] = s;
}

// one element: FP64 -> fixed point (shared scale), `slices` signed 8-bit digits, a
// level sum per digit (a stand-in for the exact integer products of that level,
// which the tensor cores would deliver), levels recombined with shifts into an
// integer and converted back to FP64
template <int S> __global__ void ozaki_elementwise_kernel(const double *x, double *y, long long n, double scale)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long q = __double2ll_rn(x[i] * scale);
        int dig[S];
#pragma unroll
        for (int l = 0; l < S; ++l) dig[l] = (int)(signed char)(q >> (8 * (S - 1 - l)));
        long long acc = 0;
#pragma unroll
        for (int l = 0; l < S; ++l) acc = (acc << 8) + (long long)dig[l] * dig[S - 1 - l];
        y[i] = __ll2double_rn(acc) * (1.0 / scale);
    }
}

struct DiagTimer {
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    DiagTimer()
    {
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    ~DiagTimer()
    {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamDestroy(st);
    }
    template <typename F> float best_ms(F &&launch, int reps)
    {
        launch();  // warm-up
        float best = 1e30f;
        for (int r = 0; r < reps; ++r) {
            cudaEventRecord(e0, st);
            launch();
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) best = ms;
        }
        return best;
    }
};

int sm_count(int *sms)
{
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return rc;
    return cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
}

// ---- how the FP64 tensor path rounds, and whether it shares the FMA pipe ----------

// pseudo-random double of mixed magnitude (exponents 2^-20 .. 2^19) from a 64-bit key
__device__ __forceinline__ double diag_value(unsigned long long key)
{
    unsigned long long z = key * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * 0x1p-53 * 2.0 - 1.0;  // [-1, 1)
    return ldexp(u, (int)((z >> 3) % 40) - 20);
}

// Every warp draws A (8x4), B (4x8) and C (8x8, zero for even tiles), runs one
// mma.sync.m8n8k4.f64 and compares each of its lane's two outputs with the ascending
// FMA chain fma(a3,b3, fma(a2,b2, fma(a1,b1, fma(a0,b0,c)))) and with the descending one.
__global__ void dmma_chain_kernel(unsigned long long *counts, int tiles_per_warp)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
    const unsigned long long warp = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    unsigned long long asc = 0, desc = 0, total = 0;
    for (int t = 0; t < tiles_per_warp; ++t) {
        const unsigned long long base = (warp * tiles_per_warp + t) * 256ull;
        auto A = [&](int r, int k) { return diag_value(base + r * 4 + k); };
        auto B = [&](int k, int c) { return diag_value(base + 64 + k * 8 + c); };
        auto C = [&](int r, int c) { return (t & 1) ? diag_value(base + 128 + r * 8 + c) : 0.0; };
        double d0 = C(g, 2 * s), d1 = C(g, 2 * s + 1);
        const double a = A(g, s), b = B(s, g);
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(d0), "+d"(d1)
                     : "d"(a), "d"(b));
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int c = 2 * s + j;
            double up = C(g, c), down = C(g, c);
            for (int k = 0; k < 4; ++k) up = fma(A(g, k), B(k, c), up);
            for (int k = 3; k >= 0; --k) down = fma(A(g, k), B(k, c), down);
            const double got = j ? d1 : d0;
            asc += got == up;
            desc += got == down;
            ++total;
        }
    }
    atomicAdd(counts + 0, asc);
    atomicAdd(counts + 1, desc);
    atomicAdd(counts + 2, total);
}

// mode 0: every warp runs DFMA chains; 1: every warp runs m8n8k4 chains; 2: even warps
// DFMA, odd warps DMMA.  Per warp and iteration both do 8 x 256 FMAs.
__global__ void fp64_mix_kernel(double *out, int iters, int mode)
{
    const int w = threadIdx.x >> 5;
    const bool mma = mode == 1 || (mode == 2 && (w & 1));
    double s = 0;
    if (mma) {
        const double a = 1.0 + 1e-9 * threadIdx.x, b = 1.0 - 1e-9 * threadIdx.x;
        double c[8][2];
#pragma unroll
        for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = j;
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                             : "+d"(c[j][0]), "+d"(c[j][1])
                             : "d"(a), "d"(b));
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1];
    } else {
        const double a = 1.0 + 1e-9 * threadIdx.x, b = 1e-9;
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = threadIdx.x + j;
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int r = 0; r < 8; ++r)  // 8 chains x 8 FMAs per lane = 8 x 256 per warp
#pragma unroll
                for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) s += x[j];
    }
    if (s == 1234.5678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int kronmult_diag_fp64_mma_gflops(double *gflops)
{
    if (!gflops) return cudaErrorInvalidValue;
    int sms = 0;
    cudaError_t rc = (cudaError_t)sm_count(&sms);
    if (rc != cudaSuccess) return rc;
    double *out = nullptr;
    if ((rc = cudaMalloc(&out, sizeof(double))) != cudaSuccess) return rc;
    const int blocks = sms * 4, threads = 256, iters = 400;
    float ms;
    {
        DiagTimer t;
        ms = t.best_ms([&] { dmma_rate_kernel<<<blocks, threads, 0, t.st>>>(out, iters); }, 3);
    }
    rc = cudaGetLastError();
    cudaFree(out);
    if (rc != cudaSuccess) return rc;
    const double flops = 512.0 * 8 * iters * ((double)blocks * threads / 32);  // per warp: 8 chains x iters x 512
    *gflops = flops / (ms * 1e-3) / 1e9;
    return cudaSuccess;
}

extern "C" int kronmult_diag_int8_mma_tops(double *tops)
{
    if (!tops) return cudaErrorInvalidValue;
    int sms = 0;
    cudaError_t rc = (cudaError_t)sm_count(&sms);
    if (rc != cudaSuccess) return rc;
    int *out = nullptr;
    if ((rc = cudaMalloc(&out, sizeof(int))) != cudaSuccess) return rc;
    const int blocks = sms * 4, threads = 256, iters = 2000;
    float ms;
    {
        DiagTimer t;
        ms = t.best_ms([&] { imma_rate_kernel<<<blocks, threads, 0, t.st>>>(out, iters); }, 3);
    }
    rc = cudaGetLastError();
    cudaFree(out);
    if (rc != cudaSuccess) return rc;
    const double ops = 8192.0 * 8 * iters * ((double)blocks * threads / 32);
    *tops = ops / (ms * 1e-3) / 1e12;
    return cudaSuccess;
}

extern "C" int kronmult_diag_ozaki_elementwise_ms(long long elements, int slices, double *ms)
{
    if (!ms || elements <= 0 || slices < 4 || slices > 8) return cudaErrorInvalidValue;
    double *x = nullptr, *y = nullptr;
    cudaError_t rc = cudaMalloc(&x, (size_t)elements * sizeof(double));
    if (rc != cudaSuccess) return rc;
    if ((rc = cudaMalloc(&y, (size_t)elements * sizeof(double))) != cudaSuccess) {
        cudaFree(x);
        return rc;
    }
    cudaMemset(x, 0x3f, (size_t)elements * sizeof(double));  // finite values near 0.5
    int sms = 0;
    sm_count(&sms);
    const unsigned grid = (unsigned)sms * 8;
    const double scale = 0x1p52;
    float best;
    {
        DiagTimer t;
        auto launch = [&] {
            switch (slices) {
            case 4: ozaki_elementwise_kernel<4><<<grid, 256, 0, t.st>>>(x, y, elements, scale); break;
            case 5: ozaki_elementwise_kernel<5><<<grid, 256, 0, t.st>>>(x, y, elements, scale); break;
            case 6: ozaki_elementwise_kernel<6><<<grid, 256, 0, t.st>>>(x, y, elements, scale); break;
            case 7: ozaki_elementwise_kernel<7><<<grid, 256, 0, t.st>>>(x, y, elements, scale); break;
            default: ozaki_elementwise_kernel<8><<<grid, 256, 0, t.st>>>(x, y, elements, scale); break;
            }
        };
        best = t.best_ms(launch, 3);
    }
    rc = cudaGetLastError();
    cudaFree(x);
    cudaFree(y);
    if (rc != cudaSuccess) return rc;
    *ms = best;
    return cudaSuccess;
}

extern "C" int kronmult_diag_fp64_mma_rounding(unsigned long long *counts)
{
    if (!counts) return cudaErrorInvalidValue;
    unsigned long long *d = nullptr;
    cudaError_t rc = cudaMalloc(&d, 3 * sizeof(unsigned long long));
    if (rc != cudaSuccess) return rc;
    cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    dmma_chain_kernel<<<64, 256>>>(d, 16);  // 512 warps x 16 tiles x 64 elements
    rc = cudaGetLastError();
    if (rc == cudaSuccess) rc = cudaMemcpy(counts, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return rc;
}

extern "C" int kronmult_diag_fp64_pipe_share(double *ms)
{
    if (!ms) return cudaErrorInvalidValue;
    int sms = 0;
    cudaError_t rc = (cudaError_t)sm_count(&sms);
    if (rc != cudaSuccess) return rc;
    double *out = nullptr;
    if ((rc = cudaMalloc(&out, sizeof(double))) != cudaSuccess) return rc;
    {
        DiagTimer t;
        for (int mode = 0; mode < 3; ++mode)
            ms[mode] = t.best_ms([&] { fp64_mix_kernel<<<sms * 2, 256, 0, t.st>>>(out, 200, mode); }, 3);
    }
    rc = cudaGetLastError();
    cudaFree(out);
    return rc;
}

