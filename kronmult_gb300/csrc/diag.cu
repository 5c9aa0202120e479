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
