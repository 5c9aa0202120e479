// Shared device/host helpers for the kronmult_gb300 kernels.
//
// Terminology (follows the reference, kronmult_gpu/kronmult.cuh:28-32):
//   d  = matrix_count, the number of Kronecker factors of an entry
//   n  = matrix_size, every factor is n x n, col-major, leading dimension matrix_stride
//   N  = n^d, the length of an entry's input and output vector
//   entry k computes output[k] += kron(A_{k,0}, ..., A_{k,d-1}) . input[k]
// The tensor view of an N-vector has d indices of size n; index d-1 is the
// fastest, so A_0 acts on the slowest index (tests/utils/kronmult_naive.h:60-61).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kgb {

// A "team" is the group of threads that processes one entry at a time.  Teams
// of 8/16/32 threads live inside one warp and synchronise with __syncwarp on
// their lane mask; larger teams are whole warps and use a named barrier (id 1+team)
// or __syncthreads when the team is the whole CTA.
struct Team {
    int size;       // threads per team
    int rank;       // thread index within the team
    int id;         // team index within the CTA
    unsigned mask;  // lane mask for sub-warp teams

    __device__ __forceinline__ Team(int team_size)
    {
        size = team_size;
        id = threadIdx.x / team_size;
        rank = threadIdx.x - id * team_size;
        if (team_size >= 32) {
            mask = 0xffffffffu;
        } else {
            unsigned lane = threadIdx.x & 31u;
            unsigned base = lane & ~(unsigned)(team_size - 1);
            mask = ((team_size == 32) ? 0xffffffffu : ((1u << team_size) - 1u)) << base;
        }
    }

    __device__ __forceinline__ void sync() const
    {
        if (size <= 32) {
            __syncwarp(mask);
        } else if (size == (int)blockDim.x) {
            __syncthreads();
        } else {
            asm volatile("bar.sync %0, %1;" ::"r"(id + 1), "r"(size) : "memory");
        }
    }
};

// output accumulation into global memory: red.global.add (an atomic addition that
// returns nothing, so no result register waits for the round trip)
template <typename T> __device__ __forceinline__ void atomic_add(T *addr, T v);
template <> __device__ __forceinline__ void atomic_add<double>(double *addr, double v)
{
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(v) : "memory");
}
template <> __device__ __forceinline__ void atomic_add<float>(float *addr, float v)
{
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(v) : "memory");
}

// streaming 16-byte load (input vectors are read exactly once)
__device__ __forceinline__ int4 ld_stream16(const void *p) { return __ldcs(reinterpret_cast<const int4 *>(p)); }

}  // namespace kgb
