// Autotuner for the forward launch shape, and the process-wide tuning cache.
//
// For a (d, n, dtype) the tuner builds a synthetic batch on the current GPU (own
// factors and inputs per entry, fan-in 8, inputs larger than L2), times every
// valid candidate (team size x entries per team) with CUDA events, keeps the
// fastest in the cache and returns it.  The forward and grouped planners use a
// cached shape whenever the caller passes no explicit tuning.  The cache can be
// saved to and loaded from a text file; entries carry the SM count of the GPU
// they were measured on and are ignored on a different one.
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include "fwd_launch.cuh"
#include "tuning.cuh"

namespace kgb {

namespace {
std::mutex g_mu;
std::map<std::tuple<int, int, int, int>, kronmult_tuning> g_cache;  // (sms, d, n, dtype)

int current_sms()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    return device_info(dev).sms;
}

template <typename T> __global__ void fill_uniform(T *p, size_t n, unsigned long long seed)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        p[i] = (T)((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
}

template <typename T, typename TO>
__global__ void build_tables(const T **mats, const T **in, TO **out, T *fac, T *x, TO *y, long long nb, int d, int n,
                             int N, int fan)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nb; k += (long long)gridDim.x * blockDim.x) {
        for (int i = 0; i < d; ++i) mats[k * d + i] = fac + (k * d + i) * (long long)n * n;
        in[k] = x + k * (long long)N;
        out[k] = y + (k / fan) * (long long)N;
    }
}

template <typename T, typename TO>
int autotune_impl(int d, int n, int dtype, int nb_sample, kronmult_tuning *best, float *best_ms)
{
    const long long Nl = pow_ll(n, d);
    if (d < 1 || n < 2 || n > 8 || Nl > (1 << 24)) return cudaErrorNotSupported;
    const int N = (int)Nl;
    long long nb = nb_sample;
    if (nb <= 0) {
        nb = (256ll << 20) / ((long long)N * sizeof(T));
        if (nb < 1024) nb = 1024;
        if (nb > (1 << 20)) nb = 1 << 20;
    }
    const int fan = 8;
    const long long n_out = (nb + fan - 1) / fan;
    T *fac = nullptr, *x = nullptr;
    TO *y = nullptr;
    void *tables = nullptr;
    cudaError_t e = cudaMalloc(&fac, sizeof(T) * (size_t)nb * d * n * n);
    if (e == cudaSuccess) e = cudaMalloc(&x, sizeof(T) * (size_t)nb * N);
    if (e == cudaSuccess) e = cudaMalloc(&y, sizeof(TO) * (size_t)n_out * N);
    if (e == cudaSuccess) e = cudaMalloc(&tables, sizeof(void *) * (size_t)nb * (d + 2));
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best_t = 1e30f;
    kronmult_tuning best_tune{};
    bool found = false;
    if (e == cudaSuccess) {
        const T **mats = reinterpret_cast<const T **>(tables);
        const T **in = mats + nb * d;
        TO **out = reinterpret_cast<TO **>(const_cast<T **>(in + nb));
        fill_uniform<T><<<1024, 256, 0, st>>>(fac, (size_t)nb * d * n * n, 1);
        fill_uniform<T><<<1024, 256, 0, st>>>(x, (size_t)nb * N, 2);
        cudaMemsetAsync(y, 0, sizeof(TO) * (size_t)n_out * N, st);
        build_tables<T, TO><<<256, 256, 0, st>>>(mats, in, out, fac, x, y, nb, d, n, N, fan);
        // FP64 n with a tensor-path kernel: that plan is a candidate too (its own shape)
        if (sizeof(T) == 8 && dmma_has_n(n)) {
            kronmult_tuning t{0, 0, 0, 0, 2};
            FwdPlan<T, TO> pl;
            if (plan_forward<T, TO>(pl, d, n, mats, n, in, out, nullptr, nb, &t) == cudaSuccess && pl.smem_path) {
                launch_plan<T, TO>(pl, st);
                for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
                    cudaEventRecord(e0, st);
                    launch_plan<T, TO>(pl, st);
                    cudaEventRecord(e1, st);
                    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best_t) {
                        best_t = ms;
                        best_tune = t;
                        found = true;
                    }
                }
            }
        }
        const int F = N / n;
        const int qcap = n <= 4 ? 8 : 4;
        for (int ts = 8; ts <= 512 && e == cudaSuccess; ts *= 2) {
            const int q = (F + ts - 1) / ts;
            if (q > qcap) continue;
            if (ts > 8 && (F + ts / 2 - 1) / (ts / 2) == 1 && ts > F) continue;  // larger teams only idle
            // staging: two slots in place (2), one slot (1), and for factors read from
            // shared memory the ping-pong buffers (3)
            const int nstage = FactorInSmemHost<T>(n) ? 3 : 2;
            for (int cand = 0; cand < 3 * nstage; ++cand) {
                const int ept = (cand % 3 == 0) ? 0 : (cand % 3 == 1 ? 2 : 8);
                const int stage = cand / 3;  // 0, 1, 2 -> prefetch 2, 1, 3
                kronmult_tuning t{ts, 0, ept, stage == 0 ? 2 : (stage == 1 ? 1 : 3), sizeof(T) == 8 ? 1 : 0};
                FwdPlan<T, TO> pl;
                if (plan_forward<T, TO>(pl, d, n, mats, n, in, out, nullptr, nb, &t) != cudaSuccess) continue;
                if (!pl.smem_path) continue;
                launch_plan<T, TO>(pl, st);
                float ms_best = 1e30f;
                for (int rep = 0; rep < 3; ++rep) {
                    cudaEventRecord(e0, st);
                    launch_plan<T, TO>(pl, st);
                    cudaEventRecord(e1, st);
                    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < ms_best) ms_best = ms;
                }
                if (e != cudaSuccess) break;
                if (ms_best < best_t) {
                    best_t = ms_best;
                    best_tune = t;
                    found = true;
                }
            }
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(fac);
    cudaFree(x);
    cudaFree(y);
    cudaFree(tables);
    if (e != cudaSuccess) return e;
    if (!found) return cudaErrorNotSupported;
    tuning_cache_store(d, n, dtype, best_tune);
    if (best) *best = best_tune;
    if (best_ms) *best_ms = best_t;
    return cudaSuccess;
}

}  // namespace

bool tuning_cache_lookup(int d, int n, int dtype, kronmult_tuning &out)
{
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_cache.empty()) return false;
    }
    const int sms = current_sms();
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(std::make_tuple(sms, d, n, dtype));
    if (it == g_cache.end()) return false;
    out = it->second;
    return true;
}

void tuning_cache_store(int d, int n, int dtype, const kronmult_tuning &t)
{
    const int sms = current_sms();
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[std::make_tuple(sms, d, n, dtype)] = t;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kronmult_autotune_forward(int matrix_count, int matrix_size, int dtype, int nb_sample, kronmult_tuning *best,
                              float *best_ms)
{
    switch (dtype) {
    case KRONMULT_DTYPE_F64: return autotune_impl<double, double>(matrix_count, matrix_size, dtype, nb_sample, best, best_ms);
    case KRONMULT_DTYPE_F32: return autotune_impl<float, float>(matrix_count, matrix_size, dtype, nb_sample, best, best_ms);
    case KRONMULT_DTYPE_F32_F64OUT:
        return autotune_impl<float, double>(matrix_count, matrix_size, dtype, nb_sample, best, best_ms);
    default: return cudaErrorInvalidValue;
    }
}

int kronmult_tuning_cache_get(int matrix_count, int matrix_size, int dtype, kronmult_tuning *out)
{
    if (!out) return cudaErrorInvalidValue;
    return tuning_cache_lookup(matrix_count, matrix_size, dtype, *out) ? cudaSuccess : cudaErrorNotReady;
}

int kronmult_tuning_cache_set(int matrix_count, int matrix_size, int dtype, const kronmult_tuning *t)
{
    if (!t || t->team_size < 0 || t->ctas_per_sm < 0 || t->entries_per_team < 0 || t->prefetch < 0 || t->prefetch > 3 ||
        t->fp64_path < 0 || t->fp64_path > 4)
        return cudaErrorInvalidValue;
    tuning_cache_store(matrix_count, matrix_size, dtype, *t);
    return cudaSuccess;
}

int kronmult_tuning_cache_clear(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache.clear();
    return cudaSuccess;
}

int kronmult_tuning_cache_save(const char *path)
{
    if (!path) return cudaErrorInvalidValue;
    FILE *f = std::fopen(path, "w");
    if (!f) return cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lk(g_mu);
    std::fprintf(f, "# kronmult_gb300 tuning cache v3: sms d n dtype team_size ctas_per_sm entries_per_team prefetch "
                    "fp64_path\n");
    for (auto &kv : g_cache)
        std::fprintf(f, "%d %d %d %d %d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
                     std::get<2>(kv.first), std::get<3>(kv.first), kv.second.team_size, kv.second.ctas_per_sm,
                     kv.second.entries_per_team, kv.second.prefetch, kv.second.fp64_path);
    std::fclose(f);
    return cudaSuccess;
}

int kronmult_tuning_cache_load(const char *path)
{
    if (!path) return cudaErrorInvalidValue;
    FILE *f = std::fopen(path, "r");
    if (!f) return cudaErrorInvalidValue;
    char line[256];
    std::lock_guard<std::mutex> lk(g_mu);
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '#') continue;
        int v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const int got = std::sscanf(line, "%d %d %d %d %d %d %d %d %d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5],
                                    &v[6], &v[7], &v[8]);
        // v2 lines (8 fields) and older (7) load with the automatic FP64 path
        if (got >= 7 && got <= 9)
            g_cache[std::make_tuple(v[0], v[1], v[2], v[3])] = kronmult_tuning{v[4], v[5], v[6], v[7], v[8]};
    }
    std::fclose(f);
    return cudaSuccess;
}

}  // extern "C"
