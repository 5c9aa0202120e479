// Drop-in C++ header for kronmult_gb300.
//
// Source-compatible with the reference's kronmult_gpu/kronmult.cuh: the same
// `kronmult_batched<T>` template (kronmult_gpu/kronmult.cuh:28-32) with explicit
// specialisations for double and float (kronmult_gpu/kronmult.cu:202-224), and
// `pow_int` (kronmult_gpu/kronmult.cuh:10).  A caller that includes this header
// instead of the reference's and links libkronmult_gb300.so instead of the
// kronmult_gpu static library needs no other change.  Semantics kept: all arrays,
// pointer arrays included, on the GPU; output[k] += kron(A_k) . input[k] with
// atomic additions into shared outputs; synchronous; the return value is the
// cudaError of the call.  Differences: arguments are validated before launch
// (cudaErrorInvalidValue), inputs are left intact whenever n^d fits in shared
// memory, and aliased inputs are allowed there.
#pragma once
#include <cuda_runtime.h>

#include "kronmult_gb300.h"

// n^power for integers (the reference's pow_int; defined inline here so that
// the header can be included from several translation units)
inline int pow_int(int const number, int const power)
{
    int r = 1;
    for (int i = 0; i < power; ++i) r *= number;
    return r;
}

template <typename T>
cudaError kronmult_batched(int const matrix_count, int const matrix_size, T const *const matrix_list_batched[],
                           int const matrix_stride, T *input_batched[], T *output_batched[],
                           T *workspace_batched[], int const nb_batch);

template <>
inline cudaError kronmult_batched<double>(int const matrix_count, int const matrix_size,
                                          double const *const matrix_list_batched[], int const matrix_stride,
                                          double *input_batched[], double *output_batched[],
                                          double *workspace_batched[], int const nb_batch)
{
    return static_cast<cudaError>(kronmult_batched_f64(matrix_count, matrix_size, matrix_list_batched,
                                                       matrix_stride, input_batched, output_batched,
                                                       workspace_batched, nb_batch));
}

template <>
inline cudaError kronmult_batched<float>(int const matrix_count, int const matrix_size,
                                         float const *const matrix_list_batched[], int const matrix_stride,
                                         float *input_batched[], float *output_batched[],
                                         float *workspace_batched[], int const nb_batch)
{
    return static_cast<cudaError>(kronmult_batched_f32(matrix_count, matrix_size, matrix_list_batched,
                                                       matrix_stride, input_batched, output_batched,
                                                       workspace_batched, nb_batch));
}
