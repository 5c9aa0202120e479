// Host-side launch planning for the forward kernels.
#pragma once
#include <climits>
#include <cstdint>
#include <mutex>
#include "dmma_kernels.cuh"
#include "fwd_kernels.cuh"
#include "pair_kernels.cuh"
#include "kronmult_gb300.h"
#include "tuning.cuh"

namespace kgb {

// per-device properties, queried once
struct DeviceInfo {
    int sms = 0;
    int max_smem_optin = 0;      // bytes of dynamic shared memory one CTA may opt into
    int smem_per_sm = 0;         // bytes of shared memory per SM
    int smem_reserved_cta = 0;   // bytes the system reserves per resident CTA
};

const DeviceInfo &device_info(int dev);

// remembers which kernels have had their dynamic shared-memory limit raised
bool ensure_smem_attr(const void *fn, size_t smem);

// resident CTAs per SM for a kernel/launch shape (cached)
int occupancy(const void *fn, int block, size_t smem);

inline long long pow_ll(int b, int e)
{
    long long r = 1;
    for (int i = 0; i < e; ++i) {
        r *= b;
        if (r > (long long)INT_MAX) return (long long)INT_MAX + 1;
    }
    return r;
}

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// host twin of FactorInSmem: an n x n factor of T does not fit the register path
template <typename T> inline bool FactorInSmemHost(int n) { return (size_t)n * n * sizeof(T) > 128; }

// Team size (power of two, 8..max_ts) for an element-mapped kernel over N outputs:
// the best lane utilisation N / (ts * ceil(N / ts)) with at most max_per outputs per
// thread; among teams within 2 % of the best, the one closest to 8 outputs per thread.
// `forced` > 0 fixes the size (grown until max_per holds).  Returns 0 if none fits.
inline int elem_team_size(int N, int max_per, int forced, int max_ts)
{
    if (forced > 0) {
        int ts = forced;
        while (ts < max_ts && (N + ts - 1) / ts > max_per) ts *= 2;
        return (N + ts - 1) / ts <= max_per ? ts : 0;
    }
    double best = -1.0;
    for (int c = 8; c <= max_ts; c *= 2) {
        const int per = (N + c - 1) / c;
        if (per <= max_per) {
            const double u = (double)N / ((double)per * c);
            if (u > best) best = u;
        }
    }
    int ts = 0, dist = 1 << 30;
    for (int c = 8; c <= max_ts; c *= 2) {
        const int per = (N + c - 1) / c;
        if (per > max_per) continue;
        const double u = (double)N / ((double)per * c);
        const int dd = per > 8 ? per - 8 : 8 - per;
        if (u >= best - 0.02 && dd < dist) {
            dist = dd;
            ts = c;
        }
    }
    return ts;
}

// Lane use of a mapping in which a team of ts threads covers `items` work items in
// rounds of ts (item = rank + j * ts), when the FP64 pipe is charged per warp
// instruction issued: in teams of a warp or more, a warp whose lanes all fall beyond
// `items` skips the round, so ceil(items / 32) warp rounds issue; sub-warp teams share
// a warp and each issues ceil(items / ts) rounds.
inline double lane_use(int items, int ts)
{
    if (ts >= 32) return (double)items / (32.0 * ((items + 31) / 32));
    return (double)items / ((double)ts * ((items + ts - 1) / ts));
}

// Margin by which the element mapping's lane use must beat the fibre mapping's before
// the FP64 planners take it (measured: equal lane use left the fibre kernels as fast or
// up to 16 % faster; d = 6, n = 3, 99 % against 95 %, is the closest case taken).
constexpr double kElemMargin = 0.03;

// FP64 mapping forced by kronmult_tuning::fp64_path: 3 = whole fibres per thread,
// 4 = one output element per thread (both on the FMA pipe); 0 otherwise.
inline int fp64_mapping(const kronmult_tuning *tune)
{
    const int p = tune ? tune->fp64_path : 0;
    return (p == 3 || p == 4) ? p : 0;
}

// largest power of two <= v (v >= 1)
inline int pow2_floor(long long v)
{
    int p = 1;
    while ((long long)p * 2 <= v) p *= 2;
    return p;
}

// A resolved forward launch.
template <typename T, typename TO> struct FwdPlan {
    FwdArgs<T, TO> args{};
    const void *fn = nullptr;
    bool smem_path = false;  // register in-place shared-memory kernel
    int use_smem = 0;        // generic kernel: shared-memory ping-pong
    dim3 grid, block;
    size_t smem = 0;
    const void *fn2 = nullptr;  // second launch (pass 2 of the two-pass path), same arguments
    dim3 grid2, block2;
    size_t smem2 = 0;
};

// Fibres per thread the two-pass path's pass-1 kernel is instantiated for, by n.
inline int split_qmax(int n) { return n <= 3 ? 8 : (n <= 7 ? 4 : 2); }

// Two-pass plan for vectors beyond shared memory (split_pass1/2_kernel): the
// largest fast part n^d1 one 256-thread team sweeps in registers, then tiles of
// L fast positions for pass 2.  Returns false where no split fits.
template <typename T, typename TO>
bool plan_split(FwdPlan<T, TO> &pl, const DeviceInfo &di)
{
    FwdArgs<T, TO> &a = pl.args;
    const int n = a.n, d = a.d;
    // FP64 stays on the one-vector global sweep: it is bound by the FP64 pipe, which
    // the two passes do not relieve (measured slower on n = 8, d = 6)
    if (sizeof(T) == 8 || n < 2 || n > 8 || d < 2 || !a.ws) return false;
    const int qm = split_qmax(n);
    constexpr int kAlign = 16 / (int)sizeof(T);
    for (int d1 = d - 1; d1 >= 1; --d1) {
        const long long C = pow_ll(n, d1), F1 = C / n, R = pow_ll(n, d - d1);
        if (F1 > 256LL * qm || R > 4096) continue;
        int ts = 8;
        while (ts < 256 && (long long)ts * qm < F1) ts *= 2;
        const int vpad = round_up((int)C, kAlign), fpad = round_up(d1 * n * n, kAlign);
        const int teams = 256 / ts;
        const size_t smem1 = (size_t)teams * 2 * (vpad + fpad) * sizeof(T);  // two staging slots
        auto f1 = split_pass1_lookup<T, TO>(n, qm);
        auto f2 = split_pass2_lookup<T, TO>(n);
        if (!f1 || !f2 || smem1 > (size_t)di.max_smem_optin) continue;
        // pass-2 tile: rows of at least 128 bytes and at least 256 (fibre, position)
        // tasks per mode, where two tiles fit in half the SM; else narrower (32 bytes
        // at least)
        const int fpad2 = round_up((d - d1) * n * n, kAlign);
        int L = 128 / (int)sizeof(T);
        while ((long long)L * (R / n) < 512 && L < 512) L *= 2;
        while (L > 32 / (int)sizeof(T) &&
               (4 * R * L + 2 * fpad2) * (long long)sizeof(T) > (long long)di.max_smem_optin / 2)
            L /= 2;
        const size_t smem2 = (size_t)(4 * R * L + 2 * fpad2) * sizeof(T);
        if (smem2 > (size_t)di.max_smem_optin) return false;
        const long long tiles = (C + L - 1) / L;
        // pass 2 sums runs of up to 64 consecutive entries per CTA while leaving ~16
        // CTAs per SM
        long long ept2 = a.nb * tiles / (16LL * di.sms);
        if (ept2 > 64) ept2 = 64;
        if (ept2 < 1) ept2 = 1;
        // pass 1: up to 8 chunks per team while leaving ~8 CTAs per SM
        long long ept1 = a.nb * R / ((long long)teams * di.sms * 8);
        if (ept1 > 8) ept1 = 8;
        if (ept1 < 1) ept1 = 1;
        const long long per_cta1 = (long long)teams * ept1;
        const long long grid1 = (a.nb * R + per_cta1 - 1) / per_cta1, grid2 = (a.nb + ept2 - 1) / ept2 * tiles;
        if (grid1 > INT_MAX || grid2 > INT_MAX) return false;
        if (!ensure_smem_attr((const void *)f1, smem1) || !ensure_smem_attr((const void *)f2, smem2)) return false;
        a.team_size = ts;
        a.teams_per_cta = teams;
        a.entries_per_team = (int)ept2;  // pass 2 only; pass 1 runs one chunk per team
        a.team_elems = 2 * (vpad + fpad);
        a.vec_pad = vpad;
        a.fac_pad = fpad;
        a.prefetch = 1;
        a.split_ept1 = (int)ept1;
        a.split_d1 = d1;
        a.split_C = (int)C;
        a.split_R = (int)R;
        a.split_L = L;
        pl.fn = (const void *)f1;
        pl.smem_path = true;
        pl.grid = dim3((unsigned)grid1);
        pl.block = dim3((unsigned)(teams * ts));
        pl.smem = smem1;
        pl.fn2 = (const void *)f2;
        pl.grid2 = dim3((unsigned)grid2);
        pl.block2 = dim3(256);
        pl.smem2 = smem2;
        return true;
    }
    return false;
}

// Whether an FP64 forward of factor size n runs on the FP64 tensor path: forced by
// tuning->fp64_path == 2, automatic (0) for n = 16 only, where the FMA pipe has only the
// generic run-time-n kernel (n <= 8 has compile-time-n FMA kernels, and n = 9..15 fill
// the 8 x 8 MMA tile too poorly: both measured faster on the FMA pipe).
inline bool dmma_wanted(int n, const kronmult_tuning *tune)
{
    const int path = tune ? tune->fp64_path : 0;
    if (!dmma_has_n(n)) return false;
    return path == 2 || (path == 0 && n == 16);
}

// FP64 tensor-path plan (fwd_dmma_kernel): one entry per team of W warps, each warp
// QT tiles of 8 fibres (W * QT * 8 >= F, at most 8 tiles per warp), the vector and the
// factors in shared memory.  False where no instantiation or shared-memory size fits.
template <typename T, typename TO>
bool plan_dmma(FwdPlan<T, TO> &pl, const DeviceInfo &di, const kronmult_tuning *tune)
{
    if constexpr (sizeof(T) != 8 || sizeof(TO) != 8) {
        return false;
    } else {
        FwdArgs<T, TO> &a = pl.args;
        const int n = a.n, d = a.d, N = a.N;
        if (d < 1 || !dmma_wanted(n, tune)) return false;
        const int F = N / n, tiles = (F + 7) / 8;
        int W = 1;
        while (W < 8 && W * 8 < tiles) W *= 2;
        const int per = (tiles + W - 1) / W;
        int qt = 1;
        while (qt < per) qt *= 2;
        const bool full = F % 8 == 0 && tiles == W * qt;
        DmmaFn fn = fwd_dmma_lookup(n, qt, full);
        if (!fn) return false;
        const int vpad = round_up(N, 2), fpad = round_up(d * n * n, 2);
        const int team_elems = vpad + fpad, ts = 32 * W;
        int teams = 256 / ts;
        while (teams > 1 && (size_t)teams * team_elems * sizeof(T) > (size_t)di.max_smem_optin) teams /= 2;
        const size_t smem = (size_t)teams * team_elems * sizeof(T);
        if (smem > (size_t)di.max_smem_optin || !ensure_smem_attr((const void *)fn, smem)) return false;
        const long long grid = (a.nb + teams - 1) / teams;
        if (grid > INT_MAX) return false;
        a.team_size = ts;
        a.teams_per_cta = teams;
        a.entries_per_team = 1;
        a.team_elems = team_elems;
        a.vec_pad = vpad;
        a.fac_pad = fpad;
        a.prefetch = 0;
        pl.fn = (const void *)fn;
        pl.smem_path = true;
        pl.grid = dim3((unsigned)grid);
        pl.block = dim3((unsigned)(teams * ts));
        pl.smem = smem;
        return true;
    }
}

// Checks arguments and fills a plan.  Returns cudaSuccess, cudaErrorInvalidValue,
// or cudaErrorNotSupported (vector too long for any path without a workspace).
template <typename T, typename TO>
int plan_forward(FwdPlan<T, TO> &pl, int d, int n, const T *const *mats, int stride, const T *const *in,
                 TO *const *out, T *const *ws, long long nb, const kronmult_tuning *tune)
{
    if (d < 0 || n < 0 || nb < 0) return cudaErrorInvalidValue;
    if (stride < (n > 0 ? n : 1)) return cudaErrorInvalidValue;
    const long long Nl = pow_ll(n, d);
    if (Nl > (long long)INT_MAX) return cudaErrorInvalidValue;
    pl.args = FwdArgs<T, TO>{};
    pl.fn = nullptr;
    pl.fn2 = nullptr;
    kronmult_tuning cached{};
    if (!tune) {
        const int code = sizeof(T) == 8 ? KRONMULT_DTYPE_F64
                                        : (sizeof(TO) == 8 ? KRONMULT_DTYPE_F32_F64OUT : KRONMULT_DTYPE_F32);
        if (tuning_cache_lookup(d, n, code, cached)) tune = &cached;
    }
    if (nb == 0 || n == 0) return cudaSuccess;  // nothing to add
    if (!in || !out || (d > 0 && !mats)) return cudaErrorInvalidValue;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);
    const int N = (int)Nl;

    FwdArgs<T, TO> &a = pl.args;
    a.mats = mats;
    a.in = in;
    a.out = out;
    a.ws = ws;
    a.nb = nb;
    a.d = d;
    a.n = n;
    a.stride = stride;
    a.N = N;

    // ---- FP64 on the tensor path (n = 7, 8, 16 unless tuned otherwise)
    if (plan_dmma<T, TO>(pl, di, tune)) return cudaSuccess;

    // ---- register in-place shared-memory path: 2 <= n <= 8, d >= 1
    if (n >= 2 && n <= 8 && d >= 1) {
        const int F = N / n;
        const int qcap = (n <= 4) ? 8 : 4;
        int ts = 8;
        if (tune && tune->team_size > 0) {
            // a forced team size grows until every thread holds at most qcap fibres
            ts = tune->team_size;
            while (ts < 512 && (F + ts - 1) / ts > qcap) ts *= 2;
        } else {
            // smallest team that leaves every thread at most ~2-4 fibres (4 for FP64
            // n = 6 too: smaller teams keep more entries in flight, measured 5-34 %
            // faster on d = 2..4)
            const int qtarget = (n <= 4 || (n == 6 && sizeof(T) == 8)) ? 4 : 2;
            while (ts < 512 && (long long)ts * qtarget < F) ts *= 2;
        }
        // One entry per team (fwd_single_kernel) unless runs are requested: measured
        // fastest for FP64, where the FP64 pipe is the bound and more resident CTAs
        // hide the staging; FP32 sums runs of 8 entries by default.
        bool single = tune && tune->entries_per_team > 0 ? tune->entries_per_team == 1 : sizeof(T) == 8;
        const int ts_runs = ts;
        if (single && ts > 256) {
            ts = 256;  // the single-entry kernel runs teams of at most 256 threads
            if ((F + ts - 1) / ts > qcap) {
                single = false;
                ts = ts_runs;
            }
        }
        const int q = (F + ts - 1) / ts;
        int qmax = 1;
        while (qmax < q) qmax *= 2;
        const bool ts_ok = (ts == 8 || ts == 16 || ts == 32 || ts == 64 || ts == 128 || ts == 256 || ts == 512);
        if (single && ts_ok && qmax <= qcap) {
            const int vpad = round_up(N, 16 / (int)sizeof(T));
            const int fpad = round_up(d * n * n, 16 / (int)sizeof(T));
            const int team_elems = vpad + fpad;
            int teams = 256 / ts;
            auto fn = fwd_single_lookup<T, TO>(n, qmax);
            // Whole fibres per thread leave (ts*q - F) of ts*q lanes idle, and the FP64 pipe
            // is charged per warp instruction whatever the number of active lanes.  FP64
            // maps output elements to threads instead (fwd_single_elem_kernel) when that
            // uses the lanes clearly better: teams are the smallest power of two that gives
            // every thread at most 4 elements (2-4 elements per thread measured 5-25 %
            // faster than 6-16 on d = 3..6, n = 3..7: shorter chains per mode), and the
            // element mapping is taken when its lane use beats the fibre mapping's by more
            // than 5 points.  Measured on 128 MB batches: d = 3, n = 6 -22 %; d = 3, n = 5
            // -24 %; d = 2, n = 4 -27 %; d = 3, n = 3 / 7 and d = 5, n = 3 -14..-17 %
            // (for odd n the baseline was an element kernel taking n at run time); where
            // the lane use is equal (d = 2, n = 6..8; d = 4, n = 4..6) the fibre kernels were
            // as fast or up to 16 % faster.
            const double fibre_util = lane_use(F, ts);
            const int fmap = fp64_mapping(tune);
            if (sizeof(T) == 8 && fmap != 3 && (fmap == 4 || !(tune && tune->team_size > 0))) {
                int tse = 8;
                if (fmap == 4 && tune->team_size > 0) {
                    tse = tune->team_size;
                    while (tse < 256 && (N + tse - 1) / tse > 8) tse *= 2;
                } else {
                    while (tse < 256 && (N + tse - 1) / tse > 4) tse *= 2;
                }
                const int per = (N + tse - 1) / tse;
                const double util_e = lane_use(N, tse);
                // at most 8 elements per thread: no spills
                if (tse <= 256 && per <= 8 && (fmap == 4 || util_e > fibre_util + kElemMargin)) {
                    int emax = 1;
                    while (emax < per) emax *= 2;
                    auto fe = fwd_single_elem_lookup<T, TO>(n, emax);
                    if (fe) {
                        fn = fe;
                        ts = tse;
                        teams = 256 / ts;
                    }
                }
            }
            size_t smem = (size_t)teams * team_elems * sizeof(T);
            if (fn && smem <= (size_t)di.max_smem_optin && ensure_smem_attr((const void *)fn, smem)) {
                long long grid = (nb + teams - 1) / teams;
                // FP64 batches of one wave or less: fewer teams per CTA so that every SM holds
                // the same number of CTAs (256 CTAs on 152 SMs would give some SMs twice the
                // entries of others: d = 3, n = 4, 8192 entries)
                if (sizeof(T) == 8 && !(tune && tune->ctas_per_sm > 0) && grid > di.sms) {
                    const int occ = occupancy((const void *)fn, teams * ts, smem);
                    if (grid <= (long long)occ * di.sms) {
                        const long long k = (grid + di.sms - 1) / di.sms;  // CTAs per SM
                        const long long t2 = (nb + k * di.sms - 1) / (k * di.sms);
                        if (t2 >= 1 && t2 < teams) {
                            teams = (int)t2;
                            smem = (size_t)teams * team_elems * sizeof(T);
                            grid = (nb + teams - 1) / teams;
                        }
                    }
                }
                if (grid <= INT_MAX) {
                    a.team_size = ts;
                    a.teams_per_cta = teams;
                    a.entries_per_team = 1;
                    a.team_elems = team_elems;
                    a.vec_pad = vpad;
                    a.fac_pad = fpad;
                    a.prefetch = 0;
                    pl.fn = (const void *)fn;
                    pl.smem_path = true;
                    pl.grid = dim3((unsigned)grid);
                    pl.block = dim3((unsigned)(teams * ts));
                    pl.smem = smem;
                    return cudaSuccess;
                }
            }
        }
        // FP32, n = 4, d = 6: three modes per shared-memory pass, a lane pair per 64-value
        // tri-fibre (fwd_tri4_kernel), one team of 128 threads per CTA, a grid of about
        // 6 entries per CTA (36864 entries: 0.207 ms; 8: 0.209 ms; one wave of CTAs with
        // equal shares of all entries: 3-6 % slower), the entries spread evenly
        if constexpr (sizeof(T) == 4) {
            const bool want_tri4 = !single && n == 4 && d == 6 && !(tune && tune->prefetch == 1) &&
                                   !(tune && tune->team_size > 0);
            if (want_tri4) {
                auto fn = fwd_pair_lookup<TO>(4, 3);
                // two staging slots and the middle buffer: 55.5 KB, 4 CTAs per SM
                const size_t smem = (size_t)(3 * kTri4Elems + 2 * kTri4Fac) * sizeof(T);
                if (fn && smem <= (size_t)di.max_smem_optin && ensure_smem_attr((const void *)fn, smem)) {
                    int per_sm = (tune && tune->ctas_per_sm > 0) ? tune->ctas_per_sm
                                                                 : occupancy((const void *)fn, 128, smem);
                    if (per_sm < 1) per_sm = 1;
                    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team : 6;
                    if (ept * di.sms * per_sm > nb * 2) ept = (nb + (long long)di.sms * per_sm - 1) / ((long long)di.sms * per_sm);
                    if (ept < 1) ept = 1;
                    const long long grid = (nb + ept - 1) / ept;
                    if (grid <= INT_MAX) {
                        a.team_size = 128;
                        a.teams_per_cta = 1;
                        a.entries_per_team = (int)((nb + grid - 1) / grid);  // the largest share
                        a.team_elems = 3 * kTri4Elems + 2 * kTri4Fac;
                        a.vec_pad = kTri4Elems;  // padded layouts (t4_in, t4_phys)
                        a.fac_pad = kTri4Fac;    // factors duplicated
                        a.prefetch = 1;
                        pl.fn = (const void *)fn;
                        pl.smem_path = true;
                        pl.grid = dim3((unsigned)grid);
                        pl.block = dim3(128);
                        pl.smem = smem;
                        return cudaSuccess;
                    }
                }
            }
        }
        // FP32, n = 8, d = 3 or 4: two modes per shared-memory pass, a lane pair per
        // 64-value bi-fibre (fwd_pair8_kernel), CTAs of 128 threads
        if constexpr (sizeof(T) == 4) {
            const bool want_pair8 = !single && n == 8 && (d == 3 || d == 4) && !(tune && tune->prefetch == 1) &&
                                    !(tune && tune->team_size > 0);
            if (want_pair8) {
                const int tsp = N / 32;  // two lanes per bi-fibre: 128 (d = 4) or 16 (d = 3)
                auto fn = fwd_pair_lookup<TO>(8, 1);
                const int vpad = p8_elems(N);  // padded layout (p8_phys)
                const int fpad = round_up(d * 64, 4);
                const int team_elems = 2 * (vpad + fpad);
                const int teams = 128 / tsp;
                const size_t smem = (size_t)teams * team_elems * sizeof(T);
                if (fn && smem <= (size_t)di.max_smem_optin && ensure_smem_attr((const void *)fn, smem)) {
                    int per_sm = (tune && tune->ctas_per_sm > 0) ? tune->ctas_per_sm
                                                                 : occupancy((const void *)fn, 128, smem);
                    if (per_sm < 1) per_sm = 1;
                    const long long total_teams = (long long)di.sms * per_sm * teams;
                    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team : 8;
                    if (ept * total_teams > nb * 2) ept = (nb + total_teams - 1) / total_teams;
                    if (ept < 1) ept = 1;
                    const long long grid = (nb + ept * teams - 1) / (ept * teams);
                    if (grid <= INT_MAX && ept <= INT_MAX) {
                        a.team_size = tsp;
                        a.teams_per_cta = teams;
                        a.entries_per_team = (int)ept;
                        a.team_elems = team_elems;
                        a.vec_pad = vpad;
                        a.fac_pad = fpad;
                        a.prefetch = 1;
                        pl.fn = (const void *)fn;
                        pl.smem_path = true;
                        pl.grid = dim3((unsigned)grid);
                        pl.block = dim3(128);
                        pl.smem = smem;
                        return cudaSuccess;
                    }
                }
            }
        }
        // FP32, n = 2 or 4, d >= 2: two modes per shared-memory pass (fwd_pair_kernel)
        if constexpr (sizeof(T) == 4) {
            const bool want_pair = !single && (n == 2 || n == 4) && d >= 2 && !(tune && tune->prefetch == 1) &&
                                   !(tune && tune->team_size > 0);
            if (want_pair) {
                const int F2 = N / (n * n);
                int tsp = 8;
                while (tsp < 256 && tsp < F2) tsp *= 2;  // one bi-fibre per thread up to 256 threads
                const int qp = (F2 + tsp - 1) / tsp;
                auto fn = qp <= 2 ? fwd_pair_lookup<TO>(n, qp <= 1 ? 1 : 2) : nullptr;
                const int vpad = round_up(N, 4);
                const int fpad = round_up(d * n * n, 4);
                const int team_elems = 2 * (vpad + fpad);
                const int teams = 256 / tsp;
                const size_t smem = (size_t)teams * team_elems * sizeof(T);
                if (fn && smem <= (size_t)di.max_smem_optin && ensure_smem_attr((const void *)fn, smem)) {
                    int per_sm = (tune && tune->ctas_per_sm > 0) ? tune->ctas_per_sm
                                                                 : occupancy((const void *)fn, teams * tsp, smem);
                    if (per_sm < 1) per_sm = 1;
                    const long long total_teams = (long long)di.sms * per_sm * teams;
                    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team : 8;
                    if (ept * total_teams > nb * 2) ept = (nb + total_teams - 1) / total_teams;
                    if (ept < 1) ept = 1;
                    const long long grid = (nb + ept * teams - 1) / (ept * teams);
                    if (grid <= INT_MAX && ept <= INT_MAX) {
                        a.team_size = tsp;
                        a.teams_per_cta = teams;
                        a.entries_per_team = (int)ept;
                        a.team_elems = team_elems;
                        a.vec_pad = vpad;
                        a.fac_pad = fpad;
                        a.prefetch = 1;
                        pl.fn = (const void *)fn;
                        pl.smem_path = true;
                        pl.grid = dim3((unsigned)grid);
                        pl.block = dim3((unsigned)(teams * tsp));
                        pl.smem = smem;
                        return cudaSuccess;
                    }
                }
            }
        }
        if (ts_ok && qmax <= qcap) {
            const int vpad = round_up(N, 16 / (int)sizeof(T));
            const int fpad = round_up(d * n * n, 16 / (int)sizeof(T));
            // two staging slots (asynchronous prefetch of the next entry) unless disabled
            // or too large for half of the SM's shared memory; FP32 with factors in
            // shared memory (n >= 6) ping-pongs between vector buffers instead (three
            // vector buffers, two factor slots)
            int prefetch = (tune && tune->prefetch == 1) ? 0 : 1;
            if ((size_t)2 * (vpad + fpad) * sizeof(T) > (size_t)di.max_smem_optin / 2) prefetch = 0;
            const bool pp_ok = FactorInSmemHost<T>(n) && (size_t)(3 * vpad + 2 * fpad) * sizeof(T) <=
                                                             (size_t)di.max_smem_optin / 2;
            // default for FP32 into FP32 outputs (measured 1.5-4.5 % faster on n = 6, 8);
            // with FP64 outputs the in-place slots measured faster
            if (pp_ok && ((tune && tune->prefetch == 3) ||
                          (sizeof(T) == 4 && sizeof(TO) == 4 && (!tune || tune->prefetch == 0))))
                prefetch = 3;
            const int team_elems = prefetch == 3 ? 3 * vpad + 2 * fpad : (prefetch ? 2 : 1) * (vpad + fpad);
            const size_t team_bytes = (size_t)team_elems * sizeof(T);
            int block = ts >= 256 ? ts : 256;
            int teams = block / ts;
            // named barriers 1..15 limit the number of multi-warp teams per CTA
            while (ts >= 64 && ts < block && teams > 15) {
                block /= 2;
                teams = block / ts;
            }
            while (teams > 1 && (size_t)teams * team_bytes > (size_t)di.max_smem_optin) {
                block /= 2;
                teams = block / ts;
            }
            if (block < 32) block = 32, teams = block / ts;
            const size_t smem = (size_t)teams * team_bytes;
            if (smem <= (size_t)di.max_smem_optin) {
                auto fn = fwd_smem_lookup<T, TO>(n, qmax);
                if (fn && ensure_smem_attr((const void *)fn, smem)) {
                    int per_sm = (tune && tune->ctas_per_sm > 0) ? tune->ctas_per_sm
                                                                 : occupancy((const void *)fn, block, smem);
                    if (per_sm < 1) per_sm = 1;
                    const long long total_teams = (long long)di.sms * per_sm * teams;
                    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team : 8;
                    if (ept * total_teams > nb * 2) ept = (nb + total_teams - 1) / total_teams;  // small batches
                    if (ept < 1) ept = 1;
                    if (ept > INT_MAX) ept = INT_MAX;
                    const long long per_cta = ept * teams;
                    const long long grid = (nb + per_cta - 1) / per_cta;
                    if (grid <= INT_MAX) {
                        a.team_size = ts;
                        a.teams_per_cta = teams;
                        a.entries_per_team = (int)ept;
                        a.team_elems = team_elems;
                        a.vec_pad = vpad;
                        a.fac_pad = fpad;
                        a.prefetch = prefetch;
                        pl.fn = (const void *)fn;
                        pl.smem_path = true;
                        pl.grid = dim3((unsigned)grid);
                        pl.block = dim3((unsigned)block);
                        pl.smem = smem;
                        return cudaSuccess;
                    }
                }
            }
        }
    }

    // ---- large vectors: two passes through the workspace (input left intact)
    if (plan_split<T, TO>(pl, di)) return cudaSuccess;

    // ---- larger still: every mode through input/workspace in global memory, FP64
    // on the tensor path where it is wanted
    if constexpr (sizeof(T) == 8 && sizeof(TO) == 8) {
        if (d >= 1 && ws && dmma_wanted(n, tune)) {
            const size_t smem_s = ((size_t)round_up(n * n, 2) + 2 * (size_t)round_up(N, 2)) * sizeof(T);
            auto fn = fwd_dmma_global_lookup(n);
            if (fn && smem_s > (size_t)di.max_smem_optin) {
                const long long grid = nb < INT_MAX ? nb : INT_MAX;  // one CTA per entry
                pl.fn = (const void *)fn;
                pl.smem_path = true;
                pl.grid = dim3((unsigned)grid);
                pl.block = dim3(512);
                pl.smem = 0;
                return cudaSuccess;
            }
        }
    }
    if (n >= 2 && n <= 8 && d >= 1 && ws) {
        const size_t smem_s = ((size_t)round_up(n * n, 2) + 2 * (size_t)round_up(N, 2)) * sizeof(T);
        if (smem_s > (size_t)di.max_smem_optin) {
            auto fn = fwd_global_lookup<T, TO>(n);
            if (fn) {
                const long long grid = nb < INT_MAX ? nb : INT_MAX;  // one CTA per entry
                pl.fn = (const void *)fn;
                pl.smem_path = true;  // same launch signature as the shared-memory kernels
                pl.grid = dim3((unsigned)grid);
                pl.block = dim3(512);
                pl.smem = 0;
                return cudaSuccess;
            }
        }
    }

    // ---- generic path
    const void *fn = fwd_generic_ptr<T, TO>();
    const size_t smem_s = ((size_t)round_up(n * n, 2) + 2 * (size_t)round_up(N, 2)) * sizeof(T);
    if (smem_s <= (size_t)di.max_smem_optin && ensure_smem_attr(fn, smem_s)) {
        pl.use_smem = 1;
        pl.smem = smem_s;
    } else {
        if (!ws) return cudaErrorNotSupported;
        pl.use_smem = 0;
        pl.smem = (size_t)round_up(n * n, 2) * sizeof(T);
        if (!ensure_smem_attr(fn, pl.smem)) return cudaErrorInvalidValue;
    }
    const int block = 256;
    int per_sm = occupancy(fn, block, pl.smem);
    if (per_sm < 1) per_sm = 1;
    long long grid = (long long)di.sms * per_sm * 4;
    if (grid > nb) grid = nb;
    pl.fn = fn;
    pl.smem_path = false;
    pl.grid = dim3((unsigned)grid);
    pl.block = dim3(block);
    return cudaSuccess;
}

template <typename T, typename TO> int launch_plan(const FwdPlan<T, TO> &pl, cudaStream_t st)
{
    if (!pl.fn) return cudaSuccess;
    if (pl.smem_path) {
        auto fn = reinterpret_cast<void (*)(const FwdArgs<T, TO>)>(const_cast<void *>(pl.fn));
        fn<<<pl.grid, pl.block, pl.smem, st>>>(pl.args);
        if (pl.fn2) {
            auto fn2 = reinterpret_cast<void (*)(const FwdArgs<T, TO>)>(const_cast<void *>(pl.fn2));
            fn2<<<pl.grid2, pl.block2, pl.smem2, st>>>(pl.args);
        }
    } else {
        auto fn = reinterpret_cast<void (*)(const FwdArgs<T, TO>, int)>(const_cast<void *>(pl.fn));
        fn<<<pl.grid, pl.block, pl.smem, st>>>(pl.args, pl.use_smem);
    }
    return (int)cudaGetLastError();
}

}  // namespace kgb
