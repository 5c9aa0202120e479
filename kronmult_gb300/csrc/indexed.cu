// Indexed forward: integer tables instead of pointer arrays.
//
// Callers such as ASGarD hold their batch as integer maps (which output vector an
// entry adds into, which factor matrices it uses) over dense factor, input and
// output arrays.  This entry point takes those maps directly: one small kernel
// turns them into the pointer arrays of the kronmult_batched interface, in
// caller-provided scratch memory and on the caller's stream, and the regular
// forward runs on them.  Nothing is allocated and nothing is synchronised, so the
// pair of launches can be captured in a CUDA graph.  (For the vector lengths this
// library targets the pointer arrays are under 1 % of the bytes the forward moves;
// a second set of index-addressed kernels would not pay for itself.)
#include <climits>
#include "fwd_launch.cuh"

namespace kgb {
namespace {

template <typename T>
__global__ void build_pointer_tables(const T *factors, long long factor_pitch, const int *factor_index,
                                     const T *inputs, long long input_pitch, const int *input_index, T *outputs,
                                     long long output_pitch, const int *output_index, int d, int nb,
                                     const T **mats, const T **in, T **out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nb;
         k += (long long)gridDim.x * blockDim.x) {
        for (int i = 0; i < d; ++i) mats[k * d + i] = factors + (long long)factor_index[k * d + i] * factor_pitch;
        in[k] = inputs + (input_index ? (long long)input_index[k] : k) * input_pitch;
        out[k] = outputs + (long long)output_index[k] * output_pitch;
    }
}

template <typename T>
int indexed_async(int d, int n, int stride, const T *factors, long long factor_pitch, const int *factor_index,
                  const T *inputs, long long input_pitch, const int *input_index, T *outputs, long long output_pitch,
                  const int *output_index, int nb, void *scratch, size_t scratch_bytes, cudaStream_t st)
{
    if (d < 0 || n < 0 || nb < 0 || stride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    if (nb == 0 || n == 0) return cudaSuccess;
    if (!factors && d > 0) return cudaErrorInvalidValue;
    if (!inputs || !outputs || !output_index || (d > 0 && !factor_index) || !scratch) return cudaErrorInvalidValue;
    if ((d > 0 && factor_pitch < (long long)stride * n) || input_pitch < 0 || output_pitch < 0)
        return cudaErrorInvalidValue;
    const size_t need = (size_t)nb * (size_t)(d + 2) * sizeof(void *);
    if (scratch_bytes < need || (reinterpret_cast<uintptr_t>(scratch) & 7u)) return cudaErrorInvalidValue;
    const T **mats = static_cast<const T **>(scratch);
    const T **in = mats + (size_t)nb * d;
    T **out = const_cast<T **>(in + nb);
    const int grid = (int)((nb + 255) / 256 < 65535 ? (nb + 255) / 256 : 65535);
    build_pointer_tables<T><<<grid, 256, 0, st>>>(factors, factor_pitch, factor_index, inputs, input_pitch,
                                                  input_index, outputs, output_pitch, output_index, d, nb, mats,
                                                  in, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    FwdPlan<T, T> pl;
    int rc = plan_forward<T, T>(pl, d, n, mats, stride, in, out, nullptr, nb, nullptr);
    if (rc != cudaSuccess) return rc;
    return launch_plan<T, T>(pl, st);
}

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" {

long long kronmult_indexed_scratch_bytes(int matrix_count, int nb_batch)
{
    if (matrix_count < 0 || nb_batch < 0) return -1;
    return (long long)nb_batch * (matrix_count + 2) * (long long)sizeof(void *);
}

int kronmult_indexed_f64_async(int matrix_count, int matrix_size, int matrix_stride, const double *factors,
                               long long factor_pitch, const int *factor_index, const double *inputs,
                               long long input_pitch, const int *input_index, double *outputs,
                               long long output_pitch, const int *output_index, int nb_batch, void *scratch,
                               long long scratch_bytes, void *stream)
{
    if (scratch_bytes < 0) return cudaErrorInvalidValue;
    return indexed_async<double>(matrix_count, matrix_size, matrix_stride, factors, factor_pitch, factor_index,
                                 inputs, input_pitch, input_index, outputs, output_pitch, output_index, nb_batch,
                                 scratch, (size_t)scratch_bytes, (cudaStream_t)stream);
}

int kronmult_indexed_f32_async(int matrix_count, int matrix_size, int matrix_stride, const float *factors,
                               long long factor_pitch, const int *factor_index, const float *inputs,
                               long long input_pitch, const int *input_index, float *outputs,
                               long long output_pitch, const int *output_index, int nb_batch, void *scratch,
                               long long scratch_bytes, void *stream)
{
    if (scratch_bytes < 0) return cudaErrorInvalidValue;
    return indexed_async<float>(matrix_count, matrix_size, matrix_stride, factors, factor_pitch, factor_index,
                                inputs, input_pitch, input_index, outputs, output_pitch, output_index, nb_batch,
                                scratch, (size_t)scratch_bytes, (cudaStream_t)stream);
}

}  // extern "C"
