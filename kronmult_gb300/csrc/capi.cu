// C ABI of kronmult_gb300 (declarations: include/kronmult_gb300.h).
#include <map>
#include <mutex>
#include <utility>
#include "fwd_launch.cuh"

namespace kgb {

const DeviceInfo &device_info(int dev)
{
    static std::mutex mu;
    static std::map<int, DeviceInfo> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    DeviceInfo di;
    cudaDeviceGetAttribute(&di.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&di.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (di.sms <= 0) di.sms = 1;
    if (di.max_smem_optin <= 0) di.max_smem_optin = 48 * 1024;
    return cache.emplace(dev, di).first->second;
}

bool ensure_smem_attr(const void *fn, size_t smem)
{
    if (smem <= 48 * 1024) return true;
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, fn);
    auto it = done.find(key);
    if (it != done.end() && it->second >= smem) return true;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    done[key] = smem;
    return true;
}

int occupancy(const void *fn, int block, size_t smem)
{
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int, size_t>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    auto key = std::make_tuple(dev, fn, block, smem);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    int nblk = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, fn, block, smem) != cudaSuccess) {
        cudaGetLastError();
        nblk = 1;
    }
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = nblk;
    return nblk;
}

template <typename T, typename TO>
static int forward_async(int d, int n, const T *const *mats, int stride, const T *const *in, TO *const *out,
                         T *const *ws, long long nb, cudaStream_t st, const kronmult_tuning *tune)
{
    FwdPlan<T, TO> pl;
    int rc = plan_forward<T, TO>(pl, d, n, mats, stride, in, out, ws, nb, tune);
    if (rc != cudaSuccess) return rc;
    return launch_plan<T, TO>(pl, st);
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kronmult_batched_f64_async(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                               int matrix_stride, double **input_batched, double **output_batched,
                               double **workspace_batched, int nb_batch, void *stream,
                               const kronmult_tuning *tuning)
{
    return forward_async<double, double>(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                         input_batched, output_batched, workspace_batched, nb_batch,
                                         (cudaStream_t)stream, tuning);
}

int kronmult_batched_f32_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                               int matrix_stride, float **input_batched, float **output_batched,
                               float **workspace_batched, int nb_batch, void *stream,
                               const kronmult_tuning *tuning)
{
    return forward_async<float, float>(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                       input_batched, output_batched, workspace_batched, nb_batch,
                                       (cudaStream_t)stream, tuning);
}

int kronmult_batched_f64(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                         int matrix_stride, double **input_batched, double **output_batched,
                         double **workspace_batched, int nb_batch)
{
    int rc = kronmult_batched_f64_async(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                        input_batched, output_batched, workspace_batched, nb_batch, nullptr,
                                        nullptr);
    if (rc != cudaSuccess) return rc;
    return (int)cudaDeviceSynchronize();
}

int kronmult_batched_f32(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                         int matrix_stride, float **input_batched, float **output_batched,
                         float **workspace_batched, int nb_batch)
{
    int rc = kronmult_batched_f32_async(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                        input_batched, output_batched, workspace_batched, nb_batch, nullptr,
                                        nullptr);
    if (rc != cudaSuccess) return rc;
    return (int)cudaDeviceSynchronize();
}

int kronmult_batched_f32_f64out_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                                      int matrix_stride, const float *const *input_batched,
                                      double *const *output_batched, float *const *workspace_batched,
                                      int nb_batch, int compute, void *stream, const kronmult_tuning *tuning)
{
    if (compute != KRONMULT_COMPUTE_FP32) return cudaErrorNotSupported;
    return forward_async<float, double>(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                        input_batched, output_batched, workspace_batched, nb_batch,
                                        (cudaStream_t)stream, tuning);
}

long long kronmult_pow_int(int number, int power) { return pow_ll(number, power); }

const char *kronmult_error_string(int status) { return cudaGetErrorString((cudaError_t)status); }

int kronmult_abi_version(void) { return KRONMULT_GB300_VERSION; }

}  // extern "C"
