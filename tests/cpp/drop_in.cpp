// A C++ caller written against the reference's interface (kronmult.cuh), built
// against include/kronmult.cuh and libkronmult_gb300.so.  It follows the flow of
// the reference's GPU test (tests/kronmult_test_gpu.cpp:14-54): device arrays and
// device pointer tables, outputs shared by consecutive entries, one call to
// kronmult_batched<T>, then a comparison with a host computation of the same
// sweep.  Prints the relative L2 error and exits non-zero above the tolerance.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "kronmult.cuh"

#define CHECK(x)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            std::fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));       \
            std::exit(2);                                                              \
        }                                                                              \
    } while (0)

template <typename T> static double run(int d, int n, int stride, int nb, int fan)
{
    const int N = pow_int(n, d);
    const int n_out = (nb + fan - 1) / fan;
    std::mt19937_64 rng(42);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::vector<T> hf((size_t)nb * d * n * stride), hx((size_t)nb * N), hy((size_t)n_out * N, T(0));
    for (auto &v : hf) v = (T)U(rng);
    for (auto &v : hx) v = (T)U(rng);
    T *df, *dx, *dy, *dw;
    CHECK(cudaMalloc(&df, sizeof(T) * hf.size()));
    CHECK(cudaMalloc(&dx, sizeof(T) * hx.size()));
    CHECK(cudaMalloc(&dy, sizeof(T) * hy.size()));
    CHECK(cudaMalloc(&dw, sizeof(T) * hx.size()));
    CHECK(cudaMemcpy(df, hf.data(), sizeof(T) * hf.size(), cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(dx, hx.data(), sizeof(T) * hx.size(), cudaMemcpyHostToDevice));
    CHECK(cudaMemset(dy, 0, sizeof(T) * hy.size()));
    std::vector<const T *> pm((size_t)nb * d);
    std::vector<T *> pin(nb), pout(nb), pws(nb);
    for (int k = 0; k < nb; ++k) {
        for (int i = 0; i < d; ++i) pm[(size_t)k * d + i] = df + ((size_t)k * d + i) * n * stride;
        pin[k] = dx + (size_t)k * N;
        pout[k] = dy + (size_t)(k / fan) * N;
        pws[k] = dw + (size_t)k * N;
    }
    const T **dpm;
    T **dpin, **dpout, **dpws;
    CHECK(cudaMalloc(&dpm, sizeof(T *) * pm.size()));
    CHECK(cudaMalloc(&dpin, sizeof(T *) * nb));
    CHECK(cudaMalloc(&dpout, sizeof(T *) * nb));
    CHECK(cudaMalloc(&dpws, sizeof(T *) * nb));
    CHECK(cudaMemcpy(dpm, pm.data(), sizeof(T *) * pm.size(), cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(dpin, pin.data(), sizeof(T *) * nb, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(dpout, pout.data(), sizeof(T *) * nb, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(dpws, pws.data(), sizeof(T *) * nb, cudaMemcpyHostToDevice));

    CHECK(kronmult_batched<T>(d, n, dpm, stride, dpin, dpout, dpws, nb));
    CHECK(cudaMemcpy(hy.data(), dy, sizeof(T) * hy.size(), cudaMemcpyDeviceToHost));

    // host sweep in double (kronmult_omp/kronmult.hpp:32-60)
    std::vector<double> ref((size_t)n_out * N, 0.0), a(N), b(N);
    for (int k = 0; k < nb; ++k) {
        for (int v = 0; v < N; ++v) a[v] = hx[(size_t)k * N + v];
        for (int i = d - 1; i >= 0; --i) {
            const T *M = hf.data() + ((size_t)k * d + i) * n * stride;
            const int F = N / n;
            for (int c = 0; c < F; ++c)
                for (int r = 0; r < n; ++r) {
                    double s = 0;
                    for (int q = 0; q < n; ++q) s += (double)M[r + q * stride] * a[q + c * n];
                    b[c + r * F] = s;
                }
            std::swap(a, b);
        }
        for (int v = 0; v < N; ++v) ref[(size_t)(k / fan) * N + v] += a[v];
    }
    double num = 0, den = 0;
    for (size_t v = 0; v < ref.size(); ++v) {
        num += (hy[v] - ref[v]) * (hy[v] - ref[v]);
        den += ref[v] * ref[v];
    }
    cudaFree(df); cudaFree(dx); cudaFree(dy); cudaFree(dw);
    cudaFree(dpm); cudaFree(dpin); cudaFree(dpout); cudaFree(dpws);
    return std::sqrt(num / den);
}

int main()
{
    const double e64 = run<double>(6, 4, 8, 90, 9);
    const double e32 = run<float>(3, 4, 67, 64, 5);
    std::printf("double d=6 n=4 stride=8: rel L2 %.3e\nfloat  d=3 n=4 stride=67: rel L2 %.3e\n", e64, e32);
    return (e64 <= 1e-13 && e32 <= 1e-5) ? 0 : 1;
}
