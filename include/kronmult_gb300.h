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
 *    vector length the fast paths cover).  Larger vectors need `workspace`: FP32
 *    ones go through it in two passes and leave `input` intact; FP64 ones (and
 *    FP32 ones beyond the two-pass limits) are processed through `input` and
 *    `workspace` in global memory, which are then clobbered as in the reference
 *    (kronmult_gpu/kronmult.cu:119-121).  `workspace_batched` may be NULL when no
 *    entry needs a global-memory path.
 *  - 0 <= n, 0 <= d, n^d <= 2^31-1, matrix_stride >= max(n, 1), nb_batch >= 0.
 */
#ifndef KRONMULT_GB300_H
#define KRONMULT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define KRONMULT_GB300_VERSION 2 /* 2: kronmult_tuning.fp64_path */

/* Compute modes for the FP32-storage entry points. */
#define KRONMULT_COMPUTE_FP32 0 /* FP32 FMA on CUDA cores */
#define KRONMULT_COMPUTE_TF32 1 /* TF32 tensor-core mode products (n == 8), FP32 accumulate */
#define KRONMULT_COMPUTE_BF16 2 /* BF16 tensor-core mode products (n == 8), FP32 accumulate */
#define KRONMULT_COMPUTE_BF16X3 3 /* split BF16 (v = hi + lo) tensor-core mode products, three MMAs
                                     (hi.hi + lo.hi + hi.lo) per product, FP32 accumulate (n == 8):
                                     about 16 significand bits per product */

/* Storage/output type codes. */
#define KRONMULT_DTYPE_F64 0        /* double factors, inputs and outputs */
#define KRONMULT_DTYPE_F32 1        /* float factors, inputs and outputs */
#define KRONMULT_DTYPE_F32_F64OUT 2 /* float factors and inputs, double outputs */
#define KRONMULT_DTYPE_F64_EMULATED 3 /* grouped plans: double factors, inputs and outputs, mode products in
                                        double-float arithmetic on the FP32 pipe (as
                                        kronmult_batched_f64_emulated_async; n = 2..8) */

/* Output modes of the grouped entry point. */
#define KRONMULT_MODE_ATOMIC 0        /* atomic additions into shared outputs */
#define KRONMULT_MODE_DETERMINISTIC 1 /* segmented reduction per output pointer, bitwise reproducible */

/* Launch shape override used by the autotuner; zero fields mean "heuristic". */
typedef struct kronmult_tuning {
    int team_size;        /* threads cooperating on one entry: 8,16,...,512 */
    int ctas_per_sm;      /* resident CTAs per SM to size the grid for (0 = occupancy; grouped
                             plans: at most this many persistent CTAs per SM); the tensor-core
                             path reserves shared memory so that at most this many CTAs are
                             resident (0 = as many as tensor memory allows) */
    int entries_per_team; /* contiguous entries one team processes (0 = one wave) */
    int prefetch;         /* 0 = automatic, 1 = one staging slot, 2 = copy the next entry asynchronously,
                             3 = as 2 with modes ping-ponging between vector buffers (n x n factors
                             over 128 bytes) */
    int fp64_path;        /* FP64 forward kernel family: 0 = automatic (the FP64 tensor path for
                             n = 16, the FP64 FMA pipe otherwise), 1 = FP64 FMA pipe, 2 = FP64
                             tensor path (mma m8n8k4; n = 6, 7, 8, 16), 3 / 4 = FMA pipe with whole
                             fibres / one output element per thread (n <= 8).  All give bitwise
                             the same k-ascending FMA chains. */
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
 * (KRONMULT_COMPUTE_*), FP64 outputs accumulated with FP64 atomics.  TF32 and
 * BF16 run the mode products on the tensor cores (tcgen05) and cover n == 8 with
 * n^d <= 4096 (cudaErrorNotSupported otherwise); FP32 covers every shape.  Same
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
 * Supports 2 <= n <= 16 with n^d small enough for one team's shared memory
 * (cudaErrorNotSupported otherwise).
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

/*
 * Grouped persistent forward (no reference counterpart; the reference serves one
 * (d, n) per call, kronmult_gpu/kronmult.cu:173-197).  Each group is one
 * kronmult_batched call's worth of arguments (device pointer tables).  A plan is
 * built once; kronmult_grouped_run then enqueues, per group, one persistent kernel
 * compiled for that group's n (2..8; n = 9..16 take n at run time) whose teams pull
 * work units from the group's device queue.  In the atomic mode the groups' kernels
 * run as parallel branches (forked from `stream` and joined back into it through
 * events); in the deterministic mode they run one after another on `stream`.  The
 * run enqueues only a memset, kernels and event waits, so it can be captured in a
 * CUDA graph.
 *
 * Deterministic mode: at plan creation every group's entries are ordered by output
 * pointer ON THE DEVICE (a sort of (pointer, entry index) pairs: equal pointers keep
 * their entry order) -- no device-to-host copy; plan creation waits for it.  A
 * segmented reduction then sums every output's entries in entry order: work units of
 * consecutive sorted entries sum their runs; an output whose entries lie in one unit
 * gets one plain read-modify-write, out + ((y_0 + y_1) + ...), and the unit pieces of
 * an output that spans units are added in order by a second kernel, out + ((s_0 +
 * s_1) + ...).  The result is bitwise reproducible for a given plan (the grouping of
 * the sums follows the unit size, tunings[g].entries_per_team, not the scheduling;
 * for n = 9..16 units are whole outputs).  If a group's pointer tables change in place,
 * kronmult_grouped_regroup re-runs that ordering on a stream (capturable too) before
 * the next run.  Outputs may be shared between groups (the groups run in order).
 *
 * Atomic mode: runs of consecutive entries with one output pointer are summed in
 * registers and added with atomics, as kronmult_batched does; the plan reads none of
 * the tables.
 *
 * Supports 2 <= n <= 16 with n^d small enough for one team's shared memory
 * (cudaErrorNotSupported otherwise).  tunings[g].team_size forces a team size,
 * tunings[g].entries_per_team the work unit (entries per queue item).
 */
typedef struct kronmult_group {
    int matrix_count, matrix_size, matrix_stride, nb_batch;
    const void *const *matrix_list_batched; /* nb*d device pointers */
    const void *const *input_batched;       /* nb device pointers */
    void *const *output_batched;            /* nb device pointers (may alias) */
} kronmult_group;

typedef struct kronmult_grouped_plan_s *kronmult_grouped_plan;

int kronmult_grouped_plan_create(kronmult_grouped_plan *plan, const kronmult_group *groups, int n_groups, int dtype,
                                 int mode, const kronmult_tuning *tunings);
int kronmult_grouped_run(kronmult_grouped_plan plan, void *stream);
/* info[0..5] = largest grid, largest block (threads per CTA, at most 256), largest dynamic shared bytes, work units (all
 * groups), kernels per run (forward groups + adjoint groups), entries ordered on the
 * device (deterministic mode) */
int kronmult_grouped_plan_info(kronmult_grouped_plan plan, long long *info, int n_info);
int kronmult_grouped_plan_destroy(kronmult_grouped_plan plan);
/* Re-runs the deterministic mode's device-side ordering of every group on `stream`
 * (after a pointer table changed in place: the deterministic run reads copies of the
 * tables in sorted order, made by this ordering); a no-op in the atomic mode. */
int kronmult_grouped_regroup(kronmult_grouped_plan plan, void *stream);

/*
 * Adjoint groups in a grouped plan (no reference counterpart): one
 * kronmult_batched_adjoint call's worth of arguments each.  A plan made with
 * kronmult_grouped_plan_create_with_adjoint runs, besides its forward groups, every
 * adjoint group with the adjoint kernel as one more parallel branch of the same run
 * (adjoint gradients are always added with atomics), so that one captured graph
 * replays a whole forward + backward step.  The adjoint does not read the forward's
 * outputs: the branches are independent.
 */
typedef struct kronmult_adjoint_group {
    int matrix_count, matrix_size, matrix_stride, nb_batch;
    const void *const *matrix_list_batched;  /* nb*d device pointers */
    const void *const *input_batched;        /* nb device pointers */
    const void *const *grad_output_batched;  /* nb device pointers (gradient of each entry's output) */
    void *const *grad_input_batched;         /* nb device pointers, or NULL */
    void *const *grad_matrix_list_batched;   /* nb*d device pointers, or NULL */
    int grad_matrix_stride;
} kronmult_adjoint_group;

int kronmult_grouped_plan_create_with_adjoint(kronmult_grouped_plan *plan, const kronmult_group *groups,
                                              int n_groups, const kronmult_adjoint_group *adjoint_groups,
                                              int n_adjoint, int dtype, int mode, const kronmult_tuning *tunings);

/*
 * Autotuner (no reference counterpart): times every valid launch shape of the
 * forward for (matrix_count, matrix_size, dtype) on a synthetic batch of
 * nb_sample entries (0 = enough to exceed L2), stores the fastest in the
 * process-wide tuning cache and returns it.  Allocates and synchronises.
 * kronmult_batched* and the grouped planner use the cache when given no tuning.
 */
int kronmult_autotune_forward(int matrix_count, int matrix_size, int dtype, int nb_sample, kronmult_tuning *best,
                              float *best_ms);
int kronmult_tuning_cache_get(int matrix_count, int matrix_size, int dtype, kronmult_tuning *out);
int kronmult_tuning_cache_set(int matrix_count, int matrix_size, int dtype, const kronmult_tuning *t);
int kronmult_tuning_cache_clear(void);
int kronmult_tuning_cache_save(const char *path);
int kronmult_tuning_cache_load(const char *path);

/*
 * Allocation-free FP64 forward (no counterpart in the reference).
 *
 * For callers that cannot call cudaMalloc where they run the product: code inside
 * an application-owned memory pool or arena, allocator-free callbacks, runtimes
 * that forbid device allocation after start-up.  The work list that the grouped
 * forward keeps in plan-allocated device memory lives here in a fixed array
 * compiled into the library (4 MiB + 256 bytes, held by every GPU that loads the
 * library until the process exits), so a call allocates nothing.
 *
 * Same result as kronmult_batched_f64 (output[k] += kron(A_k) . input[k], atomic
 * into shared outputs); inputs are not modified; every pointer array on the
 * device.  Work is handed out in pieces: a run of consecutive entries with one
 * output pointer, cut at entry indices that are multiples of 16 once the run holds
 * more than 16 entries, so that a few long runs (thousands of entries into a
 * handful of outputs) still spread over the whole GPU.  Each piece is summed in
 * entry order and added with one atomic per element, so the result is bitwise
 * reproducible when every output's entries form one contiguous run of at most 16
 * entries.
 * Limits: nb_batch <= KRONMULT_NOALLOC_MAX_ENTRIES (else cudaErrorInvalidValue);
 * 2 <= matrix_size <= 8, n^(d-1) <= 1024 (at most 4 fibres per thread of a
 * 256-thread team) and n^d fitting one team's shared memory (else
 * cudaErrorNotSupported; e.g. n = 2, d = 12 is refused).  Every call looks up the
 * array's device address in the current context (cudaGetSymbolAddress: no
 * allocation, no cached state, so a context re-created after cudaDeviceReset is
 * served correctly); make the first call on a device before any stream capture (it
 * may load the module).  All calls share the array and it keeps the last call's contents
 * (its counters are cleared at the start of every call): calls that overlap on the
 * GPU (other streams, other host threads) race and must be serialised.
 */
#define KRONMULT_NOALLOC_MAX_ENTRIES 1048576
int kronmult_batched_f64_noalloc(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                                 int matrix_stride, const double *const *input_batched,
                                 double *const *output_batched, int nb_batch, void *stream);

/* Reads (and with clear != 0 resets) the device error word of the tensor-core
 * kernels: 0 = no error; 1 = a bounded wait on an mbarrier timed out and the
 * kernel left early (its outputs are then incomplete).  No reference counterpart. */
int kronmult_device_error(int *code, int clear);

/* Diagnostic: runs one CTA that waits, with the tensor-core kernels' bounded wait and
 * a short limit, on an mbarrier that nothing arrives on; the wait runs out and records
 * error code 1, which is returned in *code (expected: 1) and then cleared.  Shows
 * that a wait that never completes ends in an error status, not a hang, and leaves
 * the context usable.  Synchronises the device.  No reference counterpart. */
int kronmult_diag_wait_selftest(int *code);

/* Diagnostic: measured FP64 FMA throughput of the current GPU in GFLOP/s (no
 * reference counterpart).  Allocates and synchronises; not for use in a graph. */
int kronmult_diag_fp64_fma_gflops(double *gflops);

/* Diagnostics: measured FP64 tensor-core (mma.sync f64) throughput in GFLOP/s and INT8
 * tensor-core (mma.sync s8) throughput in TOPS of the current GPU; and the time in ms
 * of the per-element work that an FP64 emulation by 8-bit integer slices on tensor
 * cores (the Ozaki scheme) needs outside the tensor cores on `elements` element-mode
 * products with `slices` slices (4..8): fixed-point scaling, splitting, recombination.
 * No reference counterpart.  Allocate and synchronise; not for use in a graph. */
int kronmult_diag_fp64_mma_gflops(double *gflops);
int kronmult_diag_int8_mma_tops(double *tops);
int kronmult_diag_ozaki_elementwise_ms(long long elements, int slices, double *ms);

/* Diagnostics of the FP64 tensor path (no reference counterpart; allocate and
 * synchronise).  kronmult_diag_fp64_mma_rounding: 524,288 elements of m8n8k4 .f64 MMAs
 * on operands of mixed magnitude (half with C = 0); counts[0] = elements equal to the
 * k-ascending FMA chain from C, counts[1] = equal to the descending chain, counts[2] =
 * elements.  kronmult_diag_fp64_pipe_share: ms[0] = all warps on DFMA chains, ms[1] = all
 * warps on m8n8k4 chains (the same FMA count per warp), ms[2] = half the warps each;
 * ms[2] near ms[0]/2 + ms[1]/2 means the two share one pipe. */
int kronmult_diag_fp64_mma_rounding(unsigned long long *counts);
int kronmult_diag_fp64_pipe_share(double *ms);

/*
 * FP64-accurate forward in emulated arithmetic (no reference counterpart): FP64
 * factors, inputs and outputs; every mode product in double-float (pairs of FP32,
 * exact two-product and two-sum) on the FP32 pipe, which on GB300 is ~60x the FP64
 * pipe.  Relative error a few units of 2^-47 per mode (the FP64 path's contract is
 * 1e-13 relative L2).  Per entry and per factor power-of-two scaling keeps any finite
 * input in range; values more than 2^126 below the largest of their vector or factor
 * count as zero.  Same semantics as kronmult_batched_f64_async otherwise (inputs not
 * modified).  Supports 2 <= n <= 8.  Vectors beyond one team's shared memory need
 * `workspace_batched` (N values per entry, overwritten): they run in two passes, the
 * fastest tensor indices per contiguous chunk and the rest per tile of the workspace,
 * each scaled by its own largest magnitude; without a workspace they return
 * cudaErrorNotSupported.
 */
int kronmult_batched_f64_emulated_async(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                                        int matrix_stride, const double *const *input_batched,
                                        double *const *output_batched, double *const *workspace_batched,
                                        int nb_batch, void *stream);

/*
 * Indexed forward: integer maps instead of pointer arrays (the interface form
 * named as the next step after the drop-in; no reference counterpart).
 *   entry k, mode i uses factor  factors + factor_index[k*d + i] * factor_pitch
 *   entry k reads                inputs  + (input_index ? input_index[k] : k) * input_pitch
 *   entry k adds into            outputs + output_index[k] * output_pitch
 * (all element offsets; every array device-resident).  The pointer arrays of the
 * kronmult_batched interface are built on `stream` into caller-provided `scratch`
 * of at least kronmult_indexed_scratch_bytes(d, nb) bytes, then the regular forward
 * runs; nothing is allocated or synchronised.  Inputs are not modified (vectors
 * beyond shared memory are not supported here: cudaErrorNotSupported).  As with
 * the pointer arrays of kronmult_batched, the indices are not range-checked: every
 * index must address a row inside its array.
 */
long long kronmult_indexed_scratch_bytes(int matrix_count, int nb_batch);
int kronmult_indexed_f64_async(int matrix_count, int matrix_size, int matrix_stride, const double *factors,
                               long long factor_pitch, const int *factor_index, const double *inputs,
                               long long input_pitch, const int *input_index, double *outputs,
                               long long output_pitch, const int *output_index, int nb_batch, void *scratch,
                               long long scratch_bytes, void *stream);
int kronmult_indexed_f32_async(int matrix_count, int matrix_size, int matrix_stride, const float *factors,
                               long long factor_pitch, const int *factor_index, const float *inputs,
                               long long input_pitch, const int *input_index, float *outputs,
                               long long output_pitch, const int *output_index, int nb_batch, void *scratch,
                               long long scratch_bytes, void *stream);

/*
 * Device address of page-locked host memory (cudaHostGetDevicePointer), for pointer
 * arrays whose inputs the kernels read straight from host memory over the
 * CPU-GPU link instead of copying them first (no reference counterpart).  Fails
 * (non-zero status, *device = NULL) for memory that is not page-locked and mapped.
 */
int kronmult_host_device_pointer(const void *host, void **device);

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
