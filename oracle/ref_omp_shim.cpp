/*
 * extern "C" shim over the reference's own CPU library, kronmult_omp.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference header is compiled unmodified from
 * where it lies (the include path is given by oracle/Makefile); this file only
 * adds C-linkage entry points so that tests and fixture scripts can call it.
 * A shim is needed because kronmult_omp/kronmult.hpp:11 defines the non-inline
 * `pow_int`, so the header can appear in one translation unit only.
 *
 *   ref_kronmult_batched_{f64,f32}  -> kronmult_batched<T>  kronmult_omp/kronmult.hpp:77-104
 *   ref_kronmult_naive_{f64,f32}    -> kronmult_batched_naive<T>  tests/utils/kronmult_naive.h:108-121
 *
 * The reference clobbers `input` and `workspace` (kronmult_omp/kronmult.hpp:51);
 * callers of this shim pass copies.
 */
#include "kronmult.hpp"
#include "utils/kronmult_naive.h"
#ifdef _OPENMP
#include <omp.h>
#endif


template <typename T> static T *new_array(size_t n) { return new T[n]; }

extern "C" {

int ref_kronmult_batched_f64(int d, int n, const double *const *mats, int stride, double **in, double **out,
                             double **ws, int nb)
{
    kronmult_batched<double>(d, n, mats, stride, in, out, ws, nb);
    return 0;
}

int ref_kronmult_batched_f32(int d, int n, const float *const *mats, int stride, float **in, float **out,
                             float **ws, int nb)
{
    kronmult_batched<float>(d, n, mats, stride, in, out, ws, nb);
    return 0;
}

int ref_kronmult_naive_f64(int d, int n, double **mats, int stride, double **in, double **out, int nb)
{
    kronmult_batched_naive<double>(d, n, mats, stride, in, out, nullptr, nb, new_array<double>,
                                   [](void *p) { delete[] static_cast<double *>(p); });
    return 0;
}

int ref_kronmult_naive_f32(int d, int n, float **mats, int stride, float **in, float **out, int nb)
{
    kronmult_batched_naive<float>(d, n, mats, stride, in, out, nullptr, nb, new_array<float>,
                                  [](void *p) { delete[] static_cast<float *>(p); });
    return 0;
}

/* Sets the OpenMP team size of later calls (OMP_NUM_THREADS is read only when the
 * OpenMP runtime loads, so a launcher's OMP_NUM_THREADS=1 cannot be undone through
 * the environment afterwards). */
void ref_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int ref_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
}
