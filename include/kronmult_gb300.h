/*
 * kronmult_gb300 -- C ABI of the GB300 (sm_103a) batched Kronecker-product
 * matrix-vector product.
 *
 * For every batch entry k:
 *     output[k] += kron(A_{k,0}, ..., A_{k,d-1}) . input[k]
 * with d = matrix_count, n = matrix_size, N = n^d; every factor is an n x n
 * col-major matrix with leading dimension matrix_stride; entry k's factors are
 * matrix_list_batched[k*d .. k*d+d-1].  Output pointers may alias (several
 * entries adding into one vector); the addition is atomic.
 *
 * Conventions shared by every entry point:
 *  - All arrays, INCLUDING the pointer arrays, must be device-accessible (device,
 *    managed or host-mapped memory), as in the reference
 *    (kronmult_gpu/kronmult.cuh:19, kronmult_gpu/README.md:38).
 *  - The return value is a cudaError_t value cast to int (0 = cudaSuccess).
 *    Arguments are validated on the host before any launch; an invalid argument
 *    returns cudaErrorInvalidValue (1) and launches nothing.  The reference does
 *    no validation (kronmult_gpu/kronmult.cu:173-197).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    The _async entry points only enqueue work: they neither allocate nor
 *    synchronise, so they can be captured in a CUDA graph.
 *  - Inputs are not modified when N*sizeof(T) fits in shared memory (every
 *    vector length the fast paths cover); larger vectors are processed through
 *    `input` and `workspace` in global memory, which are then clobbered as in the
 *    reference (kronmult_gpu/kronmult.cu:119-121).  `workspace_batched` may be
 *    NULL when no entry needs the global path.
 *  - 0 <= n, 0 <= d, n^d <= 2^31-1, matrix_stride >= max(n, 1), nb_batch >= 0.
 */
#ifndef KRONMULT_GB300_H
#define KRONMULT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define KRONMULT_GB300_VERSION 1

/* Compute modes for the FP32-storage entry points. */
#define KRONMULT_COMPUTE_FP32 0 /* FP32 FMA on CUDA cores */
#define KRONMULT_COMPUTE_TF32 1 /* TF32 tensor-core mode products (n == 8), FP32 accumulate */
#define KRONMULT_COMPUTE_BF16 2 /* BF16 tensor-core mode products (n == 8), FP32 accumulate */

/* Launch shape override used by the autotuner; zero fields mean "heuristic". */
typedef struct kronmult_tuning {
    int team_size;        /* threads cooperating on one entry: 8,16,...,512 */
    int ctas_per_sm;      /* resident CTAs per SM to size the grid for (0 = occupancy) */
    int entries_per_team; /* contiguous entries one team processes (0 = one wave) */
} kronmult_tuning;

/*
 * Drop-in replacement for kronmult_batched<double> / <float>
 * (reference: kronmult_gpu/kronmult.cuh:28-32, kronmult_gpu/kronmult.cu:202-224).
 * Synchronous: returns the status of cudaDeviceSynchronize() after the launch,
 * as the reference does (kronmult_gpu/kronmult.cu:196).
 */
int kronmult_batched_f64(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                         int matrix_stride, double **input_batched, double **output_batched,
                         double **workspace_batched, int nb_batch);
int kronmult_batched_f32(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                         int matrix_stride, float **input_batched, float **output_batched,
                         float **workspace_batched, int nb_batch);

/*
 * Asynchronous forms of the two calls above on `stream` (no reference
 * counterpart: the reference always uses the legacy stream and synchronises,
 * kronmult_gpu/kronmult.cu:191-196).  `tuning` may be NULL.
 */
int kronmult_batched_f64_async(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                               int matrix_stride, double **input_batched, double **output_batched,
                               double **workspace_batched, int nb_batch, void *stream,
                               const kronmult_tuning *tuning);
int kronmult_batched_f32_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                               int matrix_stride, float **input_batched, float **output_batched,
                               float **workspace_batched, int nb_batch, void *stream,
                               const kronmult_tuning *tuning);

/*
 * Reduced-precision forward: FP32 factors and inputs, contraction in `compute`
 * (KRONMULT_COMPUTE_*), FP64 outputs accumulated with FP64 atomics.  Same
 * semantics as kronmult_batched otherwise (reference: kronmult_gpu/kronmult.cu:216-224
 * is the FP32 path; the FP64 output accumulation has no reference counterpart).
 */
int kronmult_batched_f32_f64out_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                                      int matrix_stride, const float *const *input_batched,
                                      double *const *output_batched, float *const *workspace_batched,
                                      int nb_batch, int compute, void *stream, const kronmult_tuning *tuning);

/*
 * Adjoint of kronmult_batched (no reference counterpart; the reference applied
 * with transposed factors gives grad_input, kronmult_omp/kronmult.hpp:77-104):
 *   grad_input_batched[k]          += kron(A_{k,0}^T, ..., A_{k,d-1}^T) . grad_output_batched[k]
 *   grad_matrix_list_batched[k*d+i] += dL/dA_{k,i}   (n x n, col-major, ld grad_matrix_stride)
 * where grad_output_batched[k] is the gradient of the output vector entry k adds
 * into.  Entries that share a factor must share its gradient pointer; the
 * additions are atomic.  Either gradient table may be NULL to skip it.
 * Supports 2 <= n <= 8 (cudaErrorNotSupported otherwise).
 */
int kronmult_batched_adjoint_f64_async(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                                       int matrix_stride, const double *const *input_batched,
                                       const double *const *grad_output_batched, double *const *grad_input_batched,
                                       double *const *grad_matrix_list_batched, int grad_matrix_stride,
                                       int nb_batch, void *stream, const kronmult_tuning *tuning);
int kronmult_batched_adjoint_f32_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                                       int matrix_stride, const float *const *input_batched,
                                       const float *const *grad_output_batched, float *const *grad_input_batched,
                                       float *const *grad_matrix_list_batched, int grad_matrix_stride,
                                       int nb_batch, void *stream, const kronmult_tuning *tuning);

/* Diagnostic: measured FP64 FMA throughput of the current GPU in GFLOP/s (no
 * reference counterpart).  Allocates and synchronises; not for use in a graph. */
int kronmult_diag_fp64_fma_gflops(double *gflops);

/* Integer power as in the reference's pow_int (kronmult_gpu/kronmult.cuh:10), in 64 bits. */
long long kronmult_pow_int(int number, int power);

/* Human-readable text for a status returned by this library. */
const char *kronmult_error_string(int status);

/* Version of this ABI (KRONMULT_GB300_VERSION). */
int kronmult_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* KRONMULT_GB300_H */
