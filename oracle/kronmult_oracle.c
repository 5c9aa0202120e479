/*
 * CPU oracle for the batched Kronecker-product matrix-vector product.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only tests/, the smoke check and bench.py's CPU-baseline leg
 * use it, as the checker and as the timed CPU baseline.
 *
 * It is a plain-C restatement of the reference's CPU path (kronmult_omp):
 *   - kronmult_batched   kronmult_omp/kronmult.hpp:77-104  (OpenMP over entries)
 *   - kronmult           kronmult_omp/kronmult.hpp:32-60   (backward Algorithm-993 sweep)
 *   - multiply_transpose kronmult_omp/linear_algebra.hpp:102-121 (loop variant, no BLAS)
 *   - transpose          kronmult_omp/linear_algebra.hpp:78-88
 * and of the reference's naive explicit-Kronecker check
 *   - kronmult_naive     tests/utils/kronmult_naive.h:73-102
 *   - kronecker_product  tests/utils/kronmult_naive.h:47-67
 *
 * Arithmetic order follows the reference exactly: every mode product element is
 * a dot product started from 0 and summed over k ascending, modes run from the
 * last factor to the first, and the result is added into the output with an
 * atomic add per element.  The one deliberate difference: the reference uses
 * the caller's `input` and `workspace` vectors as its ping-pong buffers and so
 * clobbers them (kronmult_omp/kronmult.hpp:51); this restatement uses private
 * per-thread buffers and leaves the caller's inputs intact.  The numbers are
 * the same.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* number of OpenMP threads the default team would use (1 without OpenMP) */
int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* integer power, kronmult_omp/kronmult.hpp:11-15 (64-bit here) */
static int64_t ipow64(int64_t b, int e)
{
    int64_t r = 1;
    for (int i = 0; i < e; i++) r *= b;
    return r;
}

#define DEFINE_ORACLE(T, SUF)                                                                            \
    /* Mt = M^T with leading dimension n; M has leading dimension `stride`                            \
     * (kronmult_omp/linear_algebra.hpp:78-88) */                                                   \
    static void transpose_##SUF(const T *M, T *Mt, int n, int stride)                                  \
    {                                                                                                  \
        for (int r = 0; r < n; r++)                                                                    \
            for (int c = 0; c < n; c++) Mt[r + (int64_t)c * n] = M[c + (int64_t)r * stride];           \
    }                                                                                                  \
                                                                                                       \
    /* Y = X^T M^T, X is n x ncol (ld n), Y is ncol x n (ld ncol)                                      \
     * (kronmult_omp/linear_algebra.hpp:102-121) */                                                   \
    static void multiply_transpose_##SUF(const T *X, int64_t ncol, const T *M, int n, int stride, T *Y, \
                                         T *Mt)                                                        \
    {                                                                                                  \
        transpose_##SUF(M, Mt, n, stride);                                                             \
        for (int64_t c = 0; c < ncol; c++)                                                             \
            for (int r = 0; r < n; r++) {                                                              \
                T dot = 0;                                                                             \
                for (int k = 0; k < n; k++) dot += X[k + c * n] * Mt[k + (int64_t)r * n];              \
                Y[c + (int64_t)r * ncol] = dot;                                                        \
            }                                                                                          \
    }                                                                                                  \
                                                                                                       \
    /* one entry: backward sweep over the factors, then atomic add                                     \
     * (kronmult_omp/kronmult.hpp:32-60).  `buf0` holds a copy of the input. */                       \
    static void kronmult_one_##SUF(int d, int n, const T *const *mats, int stride, T *buf0, int64_t N, \
                                   T *out, T *buf1, T *Mt)                                             \
    {                                                                                                  \
        int64_t ncol = N / n;                                                                          \
        T *x = buf0, *y = buf1;                                                                        \
        for (int i = d - 1; i >= 0; i--) {                                                             \
            multiply_transpose_##SUF(x, ncol, mats[i], n, stride, y, Mt);                              \
            T *t = x;                                                                                  \
            x = y;                                                                                     \
            y = t;                                                                                     \
        }                                                                                              \
        for (int64_t i = 0; i < N; i++) {                                                              \
            _Pragma("omp atomic") out[i] += x[i];                                                      \
        }                                                                                              \
    }                                                                                                  \
                                                                                                       \
    /* batched entry point, kronmult_omp/kronmult.hpp:77-104.  Returns 0, or 2 on allocation failure. \
     * nthreads <= 0 uses the OpenMP default team. */                                                 \
    int oracle_kronmult_batched_##SUF(int d, int n, const T *const *mats, int stride, T *const *in,    \
                                      T *const *out, int nb, int nthreads)                             \
    {                                                                                                  \
        /* d = 0 is the empty product (N = 1): out += in, as in the reference */                     \
        if (nb <= 0 || d < 0 || n <= 0) return 0;                                                      \
        int64_t N = ipow64(n, d);                                                                      \
        int fail = 0;                                                                                  \
        int nt = nthreads > 0 ? nthreads : oracle_max_threads();                                       \
        _Pragma("omp parallel num_threads(nt)")                                                        \
        {                                                                                              \
            T *b0 = (T *)malloc(sizeof(T) * (size_t)N);                                                \
            T *b1 = (T *)malloc(sizeof(T) * (size_t)N);                                                \
            T *Mt = (T *)malloc(sizeof(T) * (size_t)n * (size_t)n);                                    \
            if (!b0 || !b1 || !Mt) {                                                                   \
                _Pragma("omp atomic write") fail = 1;                                                  \
            }                                                                                          \
            _Pragma("omp barrier")                                                                     \
            if (!fail) {                                                                               \
                _Pragma("omp for schedule(static)")                                                    \
                for (int k = 0; k < nb; k++) {                                                         \
                    memcpy(b0, in[k], sizeof(T) * (size_t)N);                                          \
                    kronmult_one_##SUF(d, n, mats + (int64_t)k * d, stride, b0, N, out[k], b1, Mt);    \
                }                                                                                      \
            }                                                                                          \
            free(b0);                                                                                  \
            free(b1);                                                                                  \
            free(Mt);                                                                                  \
        }                                                                                              \
        return fail ? 2 : 0;                                                                           \
    }                                                                                                  \
                                                                                                       \
    /* naive check: build kron(A_0..A_{d-1}) explicitly and add K x into out                           \
     * (tests/utils/kronmult_naive.h:47-67 and :73-102).  Row index of the product is                  \
     * row1*size2 + row2, so A_0 is the most significant factor.  Only for small n^d. */               \
    int oracle_kronmult_naive_##SUF(int d, int n, const T *const *mats, int stride, const T *in, T *out) \
    {                                                                                                  \
        int64_t N = ipow64(n, d);                                                                      \
        T *K = (T *)malloc(sizeof(T) * (size_t)(N * N));                                               \
        T *K2 = (T *)malloc(sizeof(T) * (size_t)(N * N));                                              \
        if (!K || !K2) {                                                                               \
            free(K);                                                                                   \
            free(K2);                                                                                  \
            return 2;                                                                                  \
        }                                                                                              \
        /* start from the 1 x 1 identity, so that d = 0 gives out += in */                             \
        int64_t s = 1;                                                                                 \
        K[0] = (T)1;                                                                                   \
        for (int m = 0; m < d; m++) {                                                                  \
            int64_t s2 = s * n;                                                                        \
            const T *A = mats[m];                                                                      \
            for (int64_t r1 = 0; r1 < s; r1++)                                                         \
                for (int r2 = 0; r2 < n; r2++)                                                         \
                    for (int64_t c1 = 0; c1 < s; c1++)                                                 \
                        for (int c2 = 0; c2 < n; c2++)                                                 \
                            K2[(r1 * n + r2) + (c1 * n + c2) * s2] =                                   \
                                K[r1 + c1 * s] * A[r2 + (int64_t)c2 * stride];                         \
            T *t = K;                                                                                  \
            K = K2;                                                                                    \
            K2 = t;                                                                                    \
            s = s2;                                                                                    \
        }                                                                                              \
        for (int64_t r = 0; r < N; r++)                                                                \
            for (int64_t c = 0; c < N; c++) out[r] += K[r + c * N] * in[c];                            \
        free(K);                                                                                       \
        free(K2);                                                                                      \
        return 0;                                                                                      \
    }

DEFINE_ORACLE(double, f64)
DEFINE_ORACLE(float, f32)
