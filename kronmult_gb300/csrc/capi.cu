// C ABI of kronmult_gb300 (declarations: include/kronmult_gb300.h).
#include <map>
#include <mutex>
#include <utility>
#include "adj_kernels.cuh"
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
    cudaDeviceGetAttribute(&di.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&di.smem_reserved_cta, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (di.sms <= 0) di.sms = 1;
    if (di.max_smem_optin <= 0) di.max_smem_optin = 48 * 1024;
    if (di.smem_per_sm <= 0) di.smem_per_sm = di.max_smem_optin;
    if (di.smem_reserved_cta < 0) di.smem_reserved_cta = 0;
    return cache.emplace(dev, di).first->second;
}

bool ensure_smem_attr(const void *fn, size_t smem)
{
    // always raised explicitly (cached): a kernel's static shared memory also counts
    // against the 48 KB default, so "dynamic <= 48 KB" alone is not safe
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

int launch_tc_forward(int kind, int d, int n, const float *const *mats, int stride, const float *const *in,
                      double *const *out, long long nb, cudaStream_t st, const kronmult_tuning *tune);

template <typename T, typename TO>
static int forward_async(int d, int n, const T *const *mats, int stride, const T *const *in, TO *const *out,
                         T *const *ws, long long nb, cudaStream_t st, const kronmult_tuning *tune)
{
    FwdPlan<T, TO> pl;
    int rc = plan_forward<T, TO>(pl, d, n, mats, stride, in, out, ws, nb, tune);
    if (rc != cudaSuccess) return rc;
    return launch_plan<T, TO>(pl, st);
}

template <typename T>
static int adjoint_async(int d, int n, const T *const *mats, int stride, const T *const *in, const T *const *gout,
                         T *const *gin, T *const *gmats, int gstride, long long nb, cudaStream_t st,
                         const kronmult_tuning *tune)
{
    if (d < 0 || n < 0 || nb < 0) return cudaErrorInvalidValue;
    if (stride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    if (gmats && gstride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    const long long Nl = pow_ll(n, d);
    if (Nl > (long long)INT_MAX) return cudaErrorInvalidValue;
    if (nb == 0 || n == 0 || (!gin && !gmats)) return cudaSuccess;
    if (!mats || !in || !gout) return cudaErrorInvalidValue;
    if (n < 2 || n > 16 || d < 1) return cudaErrorNotSupported;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);
    const int N = (int)Nl, R = N / n, P = n * n;
    int ts = 0;
    AdjFn<T> fn = nullptr;
    int slices = 1;
    if (sizeof(T) == 4 && n <= 8) {
        // FP32: fibre-mapped kernel (whole fibres in registers, compile-time n)
        ts = 8;
        if (tune && tune->team_size > 0) {
            ts = tune->team_size;
            if (ts < 8 || ts > 512 || (ts & (ts - 1))) return cudaErrorInvalidValue;
        } else {
            // up to 4 fibres per thread: smaller teams, more entries in flight per SM
            // (measured faster than 2 per thread on d = 3, n = 6)
            while (ts < 256 && ts * 4 < R) ts *= 2;
        }
        while (ts < 256 && (R + ts - 1) / ts > 4) ts *= 2;
        const int q = (R + ts - 1) / ts;
        int qmax = 1;
        while (qmax < q) qmax *= 2;
        // the fibre-mapped kernel runs teams of at most 256 threads (else element-mapped)
        if (qmax <= 4 && ts <= 256) fn = adj_fibre_lookup<T>(n, qmax);
        slices = ts / n;  // gradient contraction items: (row, slice of t)
    }
    if (!fn) {
        // element-mapped phases: pick the team whose lanes are best used over N outputs
        // (at most 16 outputs per thread); among equally good teams the largest wins
        if (tune && tune->team_size > 0 && (tune->team_size < 8 || tune->team_size > 512 ||
                                             (tune->team_size & (tune->team_size - 1))))
            return cudaErrorInvalidValue;
        ts = elem_team_size(N, 16, tune && tune->team_size > 0 ? tune->team_size : 0, 512);
        if (ts == 0) return cudaErrorNotSupported;
        int per = (N + ts - 1) / ts;
        int emax = 1;
        while (emax < per) emax *= 2;
        if (emax > 16) return cudaErrorNotSupported;
        fn = adj_lookup<T>(n, emax);
        // FP64, compile-time n: the smallest team of at least a warp that leaves each thread
        // at most 4 outputs with the same lane use (counted in issued warp rounds) runs the
        // 80-register form at 3 CTAs of 256 threads per SM instead of 2
        if (sizeof(T) == 8 && !(tune && tune->team_size > 0)) {
            int t4 = 32;
            while (t4 < 256 && (N + t4 - 1) / t4 > 4) t4 *= 2;
            const int per4 = (N + t4 - 1) / t4;
            int emax4 = 1;
            while (emax4 < per4) emax4 *= 2;
            const AdjFn<T> f4 = per4 <= 4 ? adj_occ_lookup<T>(n, emax4) : nullptr;
            if (f4 && lane_use(N, t4) >= lane_use(N, ts) - 0.02) {
                fn = f4;
                ts = t4;
                per = per4;
                emax = emax4;
            }
        }
        if (!fn) return cudaErrorNotSupported;
        // gradient contraction items (pair, slice of t): S slices cost about
        // ceil(S*P / lanes) passes of ceil(R / S) FMAs plus ceil(P / lanes) passes of S
        // additions to sum the slices (lanes = min(team, 32): the FP64 pipe is charged per
        // warp instruction); take the cheapest S, the smallest among equals
        const int lanes = ts < 32 ? ts : 32;
        long long best = -1;
        for (int S = 1; S <= R && S <= 64; ++S) {
            const long long cost = (long long)((S * P + lanes - 1) / lanes) * ((R + S - 1) / S) +
                                   (long long)((P + lanes - 1) / lanes) * S;
            if (best < 0 || cost < best) {
                best = cost;
                slices = S;
            }
        }
    }
    if (slices < 1) slices = 1;
    if (slices > R) slices = R;
    const int align = 16 / (int)sizeof(T);
    const int npad = round_up(N, align);
    auto team_elems_for = [&](int store_all) {
        const int np = store_all ? d : 3;
        const int ptr_elems = (8 * d + (int)sizeof(T) - 1) / (int)sizeof(T);
        return round_up(np * npad + npad + 2 * d * P + slices * P + 1 + ptr_elems, align);
    };
    int block = ts >= 256 ? ts : 256;
    int teams = block / ts;
    while (ts >= 64 && ts < block && teams > 15) {
        block /= 2;
        teams = block / ts;
    }
    int store_all = 1;
    size_t team_bytes = (size_t)team_elems_for(1) * sizeof(T);
    if (team_bytes > (size_t)di.max_smem_optin) {
        store_all = 0;
        team_bytes = (size_t)team_elems_for(0) * sizeof(T);
        if (team_bytes > (size_t)di.max_smem_optin) return cudaErrorNotSupported;
    }
    while (teams > 1 && (size_t)teams * team_bytes > (size_t)di.max_smem_optin) {
        block /= 2;
        teams = block / ts;
    }
    if (block < 32) block = 32, teams = block / ts;
    const size_t smem = (size_t)teams * team_bytes;
    if (!ensure_smem_attr((const void *)fn, smem)) return cudaErrorInvalidValue;
    int per_sm = (tune && tune->ctas_per_sm > 0) ? tune->ctas_per_sm : occupancy((const void *)fn, block, smem);
    if (per_sm < 1) per_sm = 1;
    const long long total_teams = (long long)di.sms * per_sm * teams;
    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team
                                                         : (nb + total_teams - 1) / total_teams;
    if (ept < 1) ept = 1;
    if (ept > INT_MAX) ept = INT_MAX;
    long long grid = (nb + ept * teams - 1) / (ept * teams);
    // more entries than team slots and no tuned run length: every slot of one full
    // wave takes an equal share (runs of ept entries left up to a quarter of the slots
    // idle: d = 3, n = 6, FP32, 16384 entries on 7296 slots)
    long long balanced = 0;
    if (!(tune && tune->entries_per_team > 0) && nb > total_teams) {
        balanced = total_teams;
        grid = (long long)di.sms * per_sm;
    }
    if (grid > INT_MAX) return cudaErrorInvalidValue;
    AdjArgs<T> a{};
    a.balanced_teams = balanced;
    a.mats = mats;
    a.in = in;
    a.gout = gout;
    a.gin = gin;
    a.gmats = gmats;
    a.nb = nb;
    a.d = d;
    a.n = n;
    a.stride = stride;
    a.gstride = gstride;
    a.N = N;
    a.team_size = ts;
    a.teams_per_cta = teams;
    a.entries_per_team = (int)ept;
    a.team_elems = (int)(team_bytes / sizeof(T));
    a.npad = npad;
    a.store_all = store_all;
    a.slices = slices;
    fn<<<(unsigned)grid, block, smem, st>>>(a);
    return (int)cudaGetLastError();
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
    if (compute == KRONMULT_COMPUTE_TF32 || compute == KRONMULT_COMPUTE_BF16 || compute == KRONMULT_COMPUTE_BF16X3) {
        if (matrix_count < 0 || matrix_size < 0 || nb_batch < 0 || matrix_stride < (matrix_size > 0 ? matrix_size : 1))
            return cudaErrorInvalidValue;
        if (nb_batch == 0) return cudaSuccess;
        if (!matrix_list_batched || !input_batched || !output_batched) return cudaErrorInvalidValue;
        return launch_tc_forward(compute, matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                 input_batched, output_batched, nb_batch, (cudaStream_t)stream, tuning);
    }
    if (compute != KRONMULT_COMPUTE_FP32) return cudaErrorInvalidValue;
    return forward_async<float, double>(matrix_count, matrix_size, matrix_list_batched, matrix_stride,
                                        input_batched, output_batched, workspace_batched, nb_batch,
                                        (cudaStream_t)stream, tuning);
}

int kronmult_batched_adjoint_f64_async(int matrix_count, int matrix_size, const double *const *matrix_list_batched,
                                       int matrix_stride, const double *const *input_batched,
                                       const double *const *grad_output_batched, double *const *grad_input_batched,
                                       double *const *grad_matrix_list_batched, int grad_matrix_stride,
                                       int nb_batch, void *stream, const kronmult_tuning *tuning)
{
    return adjoint_async<double>(matrix_count, matrix_size, matrix_list_batched, matrix_stride, input_batched,
                                 grad_output_batched, grad_input_batched, grad_matrix_list_batched,
                                 grad_matrix_stride, nb_batch, (cudaStream_t)stream, tuning);
}

int kronmult_batched_adjoint_f32_async(int matrix_count, int matrix_size, const float *const *matrix_list_batched,
                                       int matrix_stride, const float *const *input_batched,
                                       const float *const *grad_output_batched, float *const *grad_input_batched,
                                       float *const *grad_matrix_list_batched, int grad_matrix_stride,
                                       int nb_batch, void *stream, const kronmult_tuning *tuning)
{
    return adjoint_async<float>(matrix_count, matrix_size, matrix_list_batched, matrix_stride, input_batched,
                                grad_output_batched, grad_input_batched, grad_matrix_list_batched,
                                grad_matrix_stride, nb_batch, (cudaStream_t)stream, tuning);
}

long long kronmult_pow_int(int number, int power) { return pow_ll(number, power); }

const char *kronmult_error_string(int status) { return cudaGetErrorString((cudaError_t)status); }

int kronmult_abi_version(void) { return KRONMULT_GB300_VERSION; }

int kronmult_host_device_pointer(const void *host, void **device)
{
    if (!host || !device) return cudaErrorInvalidValue;
    *device = nullptr;
    return (int)cudaHostGetDevicePointer(device, const_cast<void *>(host), 0);
}

}  // extern "C"
