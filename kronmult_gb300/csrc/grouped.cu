// Grouped, persistent forward: one launch serves several groups of entries with
// different (d, n, fan-in), pulling work items from a device queue.
//
// No reference counterpart: the reference serves one (d, n) per call with one
// CTA per entry (kronmult_gpu/kronmult.cu:173-197).  Two output modes:
//  - atomic: runs of equal output pointers are summed in registers and added
//    with atomics (same semantics as kronmult_batched);
//  - deterministic: at plan time the entries of every group are ordered by output
//    pointer (a stable sort; the identity when equal pointers are already
//    contiguous) and cut into segments of equal pointer; each segment is summed
//    by one team in entry order and added with one plain read-modify-write, so
//    the result is bitwise reproducible from run to run.
// The plan holds everything in device memory, so kronmult_grouped_run is a
// memset of the two queue counters plus one kernel launch: it can be captured
// in a CUDA graph and replayed.
#include <algorithm>
#include <climits>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>
#include "fwd_launch.cuh"
#include "grouped.cuh"
#include "tuning.cuh"

namespace kgb {

// Every group runs the element-mapped team forward (runtime n): all lanes busy for
// any (d, n), and one small register footprint for the whole persistent kernel.
template <typename T, typename TO, bool DET>
__device__ __forceinline__ void grouped_dispatch(const GroupDesc &g, long long b, long long e, T *slots,
                                                 const Team &tm)
{
    const T *const *mats = reinterpret_cast<const T *const *>(g.mats);
    const T *const *in = reinterpret_cast<const T *const *>(g.in);
    TO *const *out = reinterpret_cast<TO *const *>(g.out);
    const T **ptrs = reinterpret_cast<const T **>(slots + 2 * (size_t)g.vec_pad);
#define KGB_G(EM)                                                                                      \
    case EM:                                                                                           \
        team_forward_elem_pf<T, TO, EM, DET>(mats, in, out, g.perm, g.d, g.n, g.stride, g.N, b, e, slots,       \
                                             g.vec_pad, ptrs, tm);                                      \
        break;
    switch (g.emax) {
        KGB_G(1) KGB_G(2) KGB_G(4)
    case 8:
        // FP64 teams hold at most 4 outputs per thread (80 registers, 3 CTAs per SM)
        if constexpr (sizeof(T) == 4)
            team_forward_elem_pf<T, TO, 8, DET>(mats, in, out, g.perm, g.d, g.n, g.stride, g.N, b, e, slots,
                                                g.vec_pad, ptrs, tm);
        break;
    case 16:
        if constexpr (sizeof(T) == 4)
            team_forward_elem_pf<T, TO, 16, DET>(mats, in, out, g.perm, g.d, g.n, g.stride, g.N, b, e, slots,
                                                 g.vec_pad, ptrs, tm);
        break;
    default: break;
    }
#undef KGB_G
}

template <typename T, typename TO, bool DET>
__global__ void __launch_bounds__(kGroupedBlock, sizeof(T) == 8 ? 3 : 2)
    grouped_kernel(const GroupDesc *groups, const CtaItem *items, int n_items, const TeamRange *ranges,
                   unsigned *counters)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(&counters[0], 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const CtaItem ci = items[it];
        const GroupDesc g = groups[ci.group];
        const int team_id = threadIdx.x / g.team_size;
        if (team_id < ci.count) {
            const Team tm(g.team_size);
            T *slots = reinterpret_cast<T *>(smem_raw) + (size_t)team_id * g.team_elems;
            const TeamRange r = ranges[ci.first_range + team_id];
            grouped_dispatch<T, TO, DET>(g, r.begin, r.end, slots, tm);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------

const void *grouped_kernel_ptr(int dtype, int mode)
{
    if (dtype == KRONMULT_DTYPE_F64)
        return mode == KRONMULT_MODE_DETERMINISTIC ? (const void *)grouped_kernel<double, double, true>
                                                   : (const void *)grouped_kernel<double, double, false>;
    return mode == KRONMULT_MODE_DETERMINISTIC ? (const void *)grouped_kernel<float, float, true>
                                               : (const void *)grouped_kernel<float, float, false>;
}

// Element mapping: the team whose lanes are best used over the N outputs of an
// entry; among equally good teams the one closest to 8 outputs per thread (enough
// independent FMA chains per thread, few threads per barrier).  FP64 teams hold at
// most 4 outputs per thread: the persistent kernel carries the register footprint
// of its largest variant, and 4 keeps it at 80 registers (3 CTAs per SM, measured
// 6 % faster on the four uneven groups than 8 per thread at 2 CTAs per SM).
static int team_shape(int d, int n, int elem, const kronmult_tuning *tune, int &ts, int &qmax, int &team_elems,
                      int &vec_pad, int &emax)
{
    const long long Nl = pow_ll(n, d);
    if (n < 2 || n > 16 || d < 1 || Nl > (long long)INT_MAX) return cudaErrorNotSupported;
    const int N = (int)Nl;
    ts = elem_team_size(N, elem == 8 ? 4 : 16, tune && tune->team_size > 0 ? tune->team_size : 0, kGroupedBlock);
    if (ts == 0) return cudaErrorNotSupported;
    const int per = (N + ts - 1) / ts;
    emax = 1;
    while (emax < per) emax *= 2;
    qmax = 0;
    // two slots of [vector | factors] plus two pointer slots of d+1 pointers
    const int align = 16 / elem;
    const int slot = round_up(N, align) + round_up(d * n * n, align);
    vec_pad = slot;  // elements per data slot
    team_elems = 2 * slot + round_up(2 * (d + 1) * 8 / elem, align);
    return cudaSuccess;
}

int grouped_plan_create(GroupedPlan *&out, const kronmult_group *groups, int n_groups, int dtype, int mode,
                        const kronmult_tuning *tunings)
{
    out = nullptr;
    if (n_groups < 0 || (n_groups > 0 && !groups)) return cudaErrorInvalidValue;
    if (dtype != KRONMULT_DTYPE_F64 && dtype != KRONMULT_DTYPE_F32) return cudaErrorInvalidValue;
    if (mode != KRONMULT_MODE_ATOMIC && mode != KRONMULT_MODE_DETERMINISTIC) return cudaErrorInvalidValue;
    const int elem = dtype == KRONMULT_DTYPE_F64 ? 8 : 4;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);

    auto *pl = new GroupedPlan();
    pl->dtype = dtype;
    pl->mode = mode;
    pl->device = dev;
    std::vector<GroupDesc> descs;
    std::vector<TeamRange> ranges;
    struct HostItem {
        CtaItem ci;
        double cost;
    };
    std::vector<HostItem> hitems;
    std::vector<long long> perm_all;
    std::vector<long long> perm_offset;
    size_t smem_max = 0;
    const void *fn = grouped_kernel_ptr(dtype, mode);
    int rc = cudaSuccess;

    // first pass: shapes and shared memory, to size the persistent grid
    std::vector<int> ts(n_groups), qmax(n_groups), te(n_groups), vp(n_groups), tpc(n_groups), em(n_groups);
    for (int g = 0; g < n_groups && rc == cudaSuccess; ++g) {
        const kronmult_group &G = groups[g];
        if (G.matrix_count < 0 || G.matrix_size < 0 || G.nb_batch < 0 ||
            G.matrix_stride < (G.matrix_size > 0 ? G.matrix_size : 1)) {
            rc = cudaErrorInvalidValue;
            break;
        }
        if (G.nb_batch > 0 && (!G.matrix_list_batched || !G.input_batched || !G.output_batched)) {
            rc = cudaErrorInvalidValue;
            break;
        }
        kronmult_tuning tt{};
        const kronmult_tuning *tp = (tunings && tunings[g].team_size > 0) ? &tunings[g] : nullptr;
        if (!tp && tuning_cache_lookup(G.matrix_count, G.matrix_size, dtype, tt) && tt.team_size <= kGroupedBlock)
            tp = &tt;
        if (G.nb_batch == 0) {
            ts[g] = 0;
            continue;
        }
        rc = team_shape(G.matrix_count, G.matrix_size, elem, tp, ts[g], qmax[g], te[g], vp[g], em[g]);
        if (rc != cudaSuccess) break;
        tpc[g] = kGroupedBlock / ts[g];
        while ((size_t)tpc[g] * te[g] * elem > (size_t)di.max_smem_optin && tpc[g] > 1) tpc[g] /= 2;
        if ((size_t)tpc[g] * te[g] * elem > (size_t)di.max_smem_optin) {
            rc = cudaErrorNotSupported;
            break;
        }
        smem_max = std::max(smem_max, (size_t)tpc[g] * te[g] * elem);
    }
    if (rc == cudaSuccess && !ensure_smem_attr(fn, smem_max)) rc = cudaErrorInvalidValue;
    int per_sm = 1;
    if (rc == cudaSuccess) {
        per_sm = std::max(1, occupancy(fn, kGroupedBlock, smem_max));
        pl->grid = di.sms * per_sm;
        pl->smem = smem_max;
        pl->fn = fn;
    }

    // second pass: entry order, segments, team ranges and CTA items
    std::vector<const void *> outp;
    std::map<const void *, int> owner;  // deterministic mode: output vector -> group
    for (int g = 0; g < n_groups && rc == cudaSuccess; ++g) {
        const kronmult_group &G = groups[g];
        GroupDesc gd{};
        gd.mats = G.matrix_list_batched;
        gd.in = G.input_batched;
        gd.out = G.output_batched;
        gd.perm = nullptr;
        gd.d = G.matrix_count;
        gd.n = G.matrix_size;
        gd.stride = G.matrix_stride;
        gd.N = (int)pow_ll(G.matrix_size, G.matrix_count);
        gd.team_size = ts[g];
        gd.teams_per_cta = tpc[g];
        gd.team_elems = te[g];
        gd.vec_pad = vp[g];
        gd.qmax = qmax[g];
        gd.emax = em[g];
        perm_offset.push_back(-1);
        const long long nb = G.nb_batch;
        if (nb == 0 || G.matrix_size == 0) {
            descs.push_back(gd);
            continue;
        }
        // segment boundaries (entry order after the optional sort)
        std::vector<long long> seg_start;  // start index of each segment in (permuted) order
        outp.resize((size_t)nb);
        if (cudaMemcpy(outp.data(), G.output_batched, sizeof(void *) * (size_t)nb, cudaMemcpyDefault) !=
            cudaSuccess) {
            rc = cudaErrorInvalidValue;
            cudaGetLastError();
            break;
        }
        std::vector<long long> order;
        if (mode == KRONMULT_MODE_DETERMINISTIC) {
            for (long long k = 0; k < nb; ++k) {
                auto ins = owner.emplace(outp[k], g);
                if (!ins.second && ins.first->second != g) rc = cudaErrorInvalidValue;  // shared across groups
            }
            if (rc != cudaSuccess) break;
            // contiguous already?  (every pointer value occurs in one run)
            std::vector<const void *> runs;
            for (long long k = 0; k < nb; ++k)
                if (k == 0 || outp[k] != outp[k - 1]) runs.push_back(outp[k]);
            std::vector<const void *> sorted_runs = runs;
            std::sort(sorted_runs.begin(), sorted_runs.end());
            const bool contiguous =
                std::adjacent_find(sorted_runs.begin(), sorted_runs.end()) == sorted_runs.end();
            if (!contiguous) {
                order.resize((size_t)nb);
                std::iota(order.begin(), order.end(), 0LL);
                std::stable_sort(order.begin(), order.end(),
                                 [&](long long a, long long b) { return outp[a] < outp[b]; });
                perm_offset.back() = (long long)perm_all.size();
                perm_all.insert(perm_all.end(), order.begin(), order.end());
            }
            for (long long k = 0; k < nb; ++k) {
                const void *pk = order.empty() ? outp[k] : outp[order[k]];
                const void *pp = k == 0 ? nullptr : (order.empty() ? outp[k - 1] : outp[order[k - 1]]);
                if (k == 0 || pk != pp) seg_start.push_back(k);
            }
        } else {
            for (long long k = 0; k < nb; ++k)
                if (k == 0 || outp[k] != outp[k - 1]) seg_start.push_back(k);
        }
        seg_start.push_back(nb);
        // entries per team range: about four ranges per resident team, whole segments
        const long long resident_teams = (long long)pl->grid * tpc[g];
        long long target = (nb + 4 * resident_teams - 1) / (4 * resident_teams);
        if (tunings && tunings[g].entries_per_team > 0) target = tunings[g].entries_per_team;
        if (target < 1) target = 1;
        std::vector<TeamRange> granges;
        if (mode == KRONMULT_MODE_DETERMINISTIC) {
            size_t s = 0;
            while (s + 1 < seg_start.size()) {
                const long long b = seg_start[s];
                long long e = seg_start[s + 1];
                ++s;
                while (s + 1 < seg_start.size() && e - b < target) {
                    e = seg_start[s + 1];
                    ++s;
                }
                granges.push_back({b, e});
            }
        } else {
            for (long long b = 0; b < nb; b += target) granges.push_back({b, std::min(nb, b + target)});
        }
        const double unit = (double)gd.d * gd.n * gd.N;  // FMAs per entry
        for (size_t r0 = 0; r0 < granges.size(); r0 += (size_t)tpc[g]) {
            const int cnt = (int)std::min<size_t>((size_t)tpc[g], granges.size() - r0);
            double cost = 0;
            long long maxlen = 0;
            for (int t = 0; t < cnt; ++t) maxlen = std::max(maxlen, granges[r0 + t].end - granges[r0 + t].begin);
            cost = unit * (double)maxlen;
            hitems.push_back({CtaItem{g, cnt, (long long)(ranges.size() + r0)}, cost});
        }
        ranges.insert(ranges.end(), granges.begin(), granges.end());
        descs.push_back(gd);
    }
    if (rc != cudaSuccess) {
        delete pl;
        return rc;
    }
    // largest items first: the queue then balances the tail
    std::stable_sort(hitems.begin(), hitems.end(), [](const HostItem &a, const HostItem &b) { return a.cost > b.cost; });
    std::vector<CtaItem> items;
    items.reserve(hitems.size());
    for (auto &h : hitems) items.push_back(h.ci);
    pl->n_items = (int)items.size();
    pl->n_groups = n_groups;

    // device copies: [counters | groups | items | ranges | perm]
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t off_cnt = 0;
    const size_t off_grp = align(off_cnt + 4 * sizeof(unsigned));
    const size_t off_itm = align(off_grp + descs.size() * sizeof(GroupDesc));
    const size_t off_rng = align(off_itm + items.size() * sizeof(CtaItem));
    const size_t off_prm = align(off_rng + ranges.size() * sizeof(TeamRange));
    const size_t total = align(off_prm + perm_all.size() * sizeof(long long));
    if (cudaMalloc(&pl->dmem, total) != cudaSuccess) {
        cudaGetLastError();
        delete pl;
        return cudaErrorMemoryAllocation;
    }
    pl->dmem_bytes = total;
    char *base = static_cast<char *>(pl->dmem);
    long long *dperm = reinterpret_cast<long long *>(base + off_prm);
    for (size_t g = 0; g < descs.size(); ++g)
        if (perm_offset[g] >= 0) descs[g].perm = dperm + perm_offset[g];
    pl->counters = reinterpret_cast<unsigned *>(base + off_cnt);
    pl->groups = reinterpret_cast<GroupDesc *>(base + off_grp);
    pl->items = reinterpret_cast<CtaItem *>(base + off_itm);
    pl->ranges = reinterpret_cast<TeamRange *>(base + off_rng);
    cudaError_t e = cudaMemset(pl->counters, 0, 4 * sizeof(unsigned));
    if (e == cudaSuccess && !descs.empty())
        e = cudaMemcpy(pl->groups, descs.data(), descs.size() * sizeof(GroupDesc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpy(pl->items, items.data(), items.size() * sizeof(CtaItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !ranges.empty())
        e = cudaMemcpy(pl->ranges, ranges.data(), ranges.size() * sizeof(TeamRange), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !perm_all.empty())
        e = cudaMemcpy(dperm, perm_all.data(), perm_all.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(pl->dmem);
        delete pl;
        return e;
    }
    pl->n_ranges = (long long)ranges.size();
    pl->n_perm = (long long)perm_all.size();
    out = pl;
    return cudaSuccess;
}

int grouped_run(const GroupedPlan *pl, cudaStream_t st)
{
    if (!pl) return cudaErrorInvalidValue;
    if (pl->n_items == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(pl->counters, 0, 4 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (pl->dtype == KRONMULT_DTYPE_F64) {
        auto fn = reinterpret_cast<void (*)(const GroupDesc *, const CtaItem *, int, const TeamRange *, unsigned *)>(
            const_cast<void *>(pl->fn));
        fn<<<pl->grid, kGroupedBlock, pl->smem, st>>>(pl->groups, pl->items, pl->n_items, pl->ranges, pl->counters);
    } else {
        auto fn = reinterpret_cast<void (*)(const GroupDesc *, const CtaItem *, int, const TeamRange *, unsigned *)>(
            const_cast<void *>(pl->fn));
        fn<<<pl->grid, kGroupedBlock, pl->smem, st>>>(pl->groups, pl->items, pl->n_items, pl->ranges, pl->counters);
    }
    return (int)cudaGetLastError();
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kronmult_grouped_plan_create(kronmult_grouped_plan *plan, const kronmult_group *groups, int n_groups, int dtype,
                                 int mode, const kronmult_tuning *tunings)
{
    if (!plan) return cudaErrorInvalidValue;
    GroupedPlan *pl = nullptr;
    int rc = grouped_plan_create(pl, groups, n_groups, dtype, mode, tunings);
    *plan = reinterpret_cast<kronmult_grouped_plan>(pl);
    return rc;
}

int kronmult_grouped_run(kronmult_grouped_plan plan, void *stream)
{
    return grouped_run(reinterpret_cast<const GroupedPlan *>(plan), (cudaStream_t)stream);
}

int kronmult_grouped_plan_info(kronmult_grouped_plan plan, long long *info, int n_info)
{
    auto *pl = reinterpret_cast<const GroupedPlan *>(plan);
    if (!pl || !info) return cudaErrorInvalidValue;
    const long long v[6] = {pl->grid, kGroupedBlock, (long long)pl->smem, pl->n_items, pl->n_ranges, pl->n_perm};
    for (int i = 0; i < n_info && i < 6; ++i) info[i] = v[i];
    return cudaSuccess;
}

int kronmult_grouped_plan_destroy(kronmult_grouped_plan plan)
{
    auto *pl = reinterpret_cast<GroupedPlan *>(plan);
    if (!pl) return cudaSuccess;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != pl->device) cudaSetDevice(pl->device);
    cudaError_t e = cudaFree(pl->dmem);
    if (dev != pl->device) cudaSetDevice(dev);
    delete pl;
    return e;
}

}  // extern "C"
