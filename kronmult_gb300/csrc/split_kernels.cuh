// Forward kernels for FP32 vectors beyond shared memory: two passes through the
// workspace (the declarations of their lookups live in fwd_kernels.cuh; the
// instantiation units that serve FP32 storage include this file).
#pragma once
#include "fwd_kernels.cuh"

namespace kgb {

// ---- large vectors: two passes over global memory (compile-time n) ---------
//
// Write N = n^d as R x C with C = n^d1 (the d1 fastest tensor indices) and
// R = n^d2, d2 = d - d1.  The backward sweep's first d1 modes (A_{d-1} .. A_{d2})
// act on the fastest index and therefore only within each contiguous chunk of C
// values; its last d2 modes (A_{d2-1} .. A_0) act only within the R values that
// share a fast position (stride C).  Pass 1 sweeps every chunk in shared memory
// with the first d1 factors and stores it to the entry's workspace; pass 2 loads
// tiles of L consecutive fast positions for all R slow positions, applies the last
// d2 factors and adds into the output with atomics.  Every value comes from the
// same k-ascending FMA chain, in the same mode order, as the one-vector sweep, so
// the result per entry is the reference kernel's bit for bit.  The input is only
// read (the reference overwrites it, kronmult_gpu/kronmult.cu:119-121); the
// workspace is overwritten.  Global traffic per entry: N read + N written (pass 1),
// N read + N added (pass 2), instead of 2N per mode.  Used for FP32 storage, where
// that traffic is the bound; FP64 stays on the global sweep, bound by its FP64
// pipe.

// Pass 1: each team sweeps a range of (entry, chunk) units with the register
// in-place sweep of the shared-memory kernels over d1 modes, two staging slots
// (the next unit's chunk and factors copied by cp.async while the current one is
// computed); results are stored to the workspace.
template <typename T, typename TO, int NN, int QMAX>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3) split_pass1_kernel(const FwdArgs<T, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    T *buf = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    T *fac = buf + a.vec_pad;
    T *buf2 = fac + a.fac_pad;
    T *fac2 = buf2 + a.vec_pad;
    const long long units = a.nb * (long long)a.split_R;
    const long long w_begin = ((long long)blockIdx.x * a.teams_per_cta + tm.id) * a.split_ept1;
    if (w_begin >= units) return;
    const long long w_end = min(w_begin + (long long)a.split_ept1, units);
    const int C = a.split_C, F = C / NN, d1 = a.split_d1, d2 = a.d - d1;
    constexpr bool kSwz = VecSwizzle<T, NN>::on;
    auto stage = [&](long long w, T *b, T *f) {
        const long long e = w / a.split_R;
        const size_t off = (size_t)(w - e * a.split_R) * (size_t)C;
        stage_async<T, NN, kSwz>(b, f, a.in[e] + off, a.mats + e * a.d + d2, C, d1, a.stride, tm);
    };
    stage(w_begin, buf, fac);
    for (long long w = w_begin; w < w_end; ++w) {
        cp_async_wait_all();
        tm.sync();  // chunk w staged for the whole team; every read of the other slot done
        if (w + 1 < w_end) stage(w + 1, buf2, fac2);
        T y[QMAX][NN];
        for (int i = d1 - 1; i >= 0; --i) {
            const T *M = fac + i * NN * NN;
            mode_team<T, NN, QMAX, kSwz, !FactorInSmem<T, NN>::value>(buf, M, M, F, tm, y);
            if (i > 0) {
                tm.sync();
#pragma unroll
                for (int q = 0; q < QMAX; ++q) {
                    const int c = tm.rank + q * tm.size;
                    if (c < F) {
#pragma unroll
                        for (int r = 0; r < NN; ++r) buf[vec_pos<T, kSwz>(c + r * F)] = y[q][r];
                    }
                }
                tm.sync();
            }
        }
        const long long e = w / a.split_R;
        T *dst = a.ws[e] + (size_t)(w - e * a.split_R) * (size_t)C;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int c = tm.rank + q * tm.size;
            if (c < F) {
#pragma unroll
                for (int r = 0; r < NN; ++r) dst[c + r * F] = y[q][r];
            }
        }
        T *t = buf;
        buf = buf2;
        buf2 = t;
        t = fac;
        fac = fac2;
        fac2 = t;
    }
    cp_async_wait_all();
}

// Pass 2: one CTA per (tile of L fast positions, range of entries).  The tile is
// held as R rows of L values (row h = workspace[h*C + l0 .. + L)), so thread
// (fibre c, column l) reads its fibre's NN values L apart and consecutive lanes
// touch consecutive words.  The next entry's tile and factors are copied
// asynchronously (cp.async) while the current one is computed; the modes
// ping-pong between the loaded tile and a scratch tile.  The last mode sums
// consecutive entries with the same output in an accumulator tile (each position
// is owned by one thread, so the sum needs no barrier) and a run is flushed with
// atomic adds along rows of L consecutive output addresses.
template <typename T, int NN>
__device__ __forceinline__ void split_tile_async(T *X, T *fac, const T *src, const T *const *mats, int R, int L,
                                                 int C, int lw, int d2, int stride)
{
    constexpr int per = 16 / (int)sizeof(T);
    if (lw == L && (L % per) == 0 && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) &&
        (((size_t)C * sizeof(T)) & 15u) == 0) {
        const int cpr = L / per;  // 16-byte chunks per row
        for (int idx = threadIdx.x; idx < R * cpr; idx += blockDim.x) {
            const int h = idx / cpr, j = idx - h * cpr;
            cp_async<16>(X + h * L + j * per, src + (size_t)h * C + j * per);
        }
    } else {
        for (int idx = threadIdx.x; idx < R * L; idx += blockDim.x) {
            const int h = idx / L, l = idx - h * L;
            if (l < lw) {
                cp_async<(int)sizeof(T)>(X + idx, src + (size_t)h * C + l);
            } else {
                X[idx] = T(0);
            }
        }
    }
    constexpr int NN2 = NN * NN;
    for (int idx = threadIdx.x; idx < d2 * NN2; idx += blockDim.x) {
        const int i = idx / NN2, rem = idx - i * NN2, k = rem / NN, r = rem - k * NN;
        cp_async<(int)sizeof(T)>(fac + idx, mats[i] + r + (size_t)k * stride);
    }
    cp_async_commit();
}

template <typename T, typename TO, int NN>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) split_pass2_kernel(const FwdArgs<T, TO> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int R = a.split_R, L = a.split_L, C = a.split_C, d2 = a.d - a.split_d1, F = R / NN;
    const int tiles = (C + L - 1) / L;
    constexpr int kAlign = 16 / (int)sizeof(T);
    const int fpad = (d2 * NN * NN + kAlign - 1) / kAlign * kAlign;
    // two factor slots, then four R x L tiles: loaded, prefetched, scratch, accumulator
    T *fac0 = reinterpret_cast<T *>(smem_raw);
    T *fac1 = fac0 + fpad;
    T *Xa = fac1 + fpad;
    T *Xb = Xa + R * L;
    T *Xc = Xb + R * L;
    T *acc = Xc + R * L;
    const int l0 = (int)(blockIdx.x % tiles) * L;
    const int lw = min(L, C - l0);
    const long long e_begin = (long long)(blockIdx.x / tiles) * a.entries_per_team;
    const long long e_end = min(e_begin + (long long)a.entries_per_team, a.nb);
    TO *cur = nullptr;
    auto flush = [&](TO *dst) {
        for (int t = threadIdx.x; t < F * L; t += blockDim.x) {
            const int c = t / L, l = t - c * L;
            if (l < lw) {
#pragma unroll
                for (int r = 0; r < NN; ++r)
                    atomic_add<TO>(dst + (size_t)(c + r * F) * C + l0 + l, (TO)acc[(c + r * F) * L + l]);
            }
        }
    };
    if (e_begin < e_end)
        split_tile_async<T, NN>(Xa, fac0, a.ws[e_begin] + l0, a.mats + e_begin * a.d, R, L, C, lw, d2, a.stride);
    for (long long e = e_begin; e < e_end; ++e) {
        TO *o = a.out[e];
        T *fac = ((e - e_begin) & 1) ? fac1 : fac0;
        cp_async_wait_all();
        __syncthreads();  // tile and factors of e complete; entry e-1 done with Xb and the other slot
        if (e + 1 < e_end)
            split_tile_async<T, NN>(Xb, ((e - e_begin) & 1) ? fac0 : fac1, a.ws[e + 1] + l0, a.mats + (e + 1) * a.d,
                                    R, L, C, lw, d2, a.stride);
        const bool fresh = o != cur;
        if (fresh && cur != nullptr) flush(cur);
        cur = o;
        T *S = Xa, *D = Xc;
        for (int i = d2 - 1; i >= 0; --i) {
            const T *M = fac + i * NN * NN;
            for (int t = threadIdx.x; t < F * L; t += blockDim.x) {
                const int c = t / L, l = t - c * L;
                T xv[NN], yv[NN];
#pragma unroll
                for (int k = 0; k < NN; ++k) xv[k] = S[(k + c * NN) * L + l];
                mode_fibre_smem<T, NN>(M, xv, yv);
                if (i > 0) {
#pragma unroll
                    for (int r = 0; r < NN; ++r) D[(c + r * F) * L + l] = yv[r];
                } else {
#pragma unroll
                    for (int r = 0; r < NN; ++r) {
                        T &s = acc[(c + r * F) * L + l];
                        s = fresh ? yv[r] : s + yv[r];
                    }
                }
            }
            if (i > 0) {
                __syncthreads();
                T *t = S;
                S = D;
                D = t;
            }
        }
        T *t = Xa;  // the prefetched tile becomes the loaded one
        Xa = Xb;
        Xb = t;
    }
    if (cur != nullptr) flush(cur);
    cp_async_wait_all();
}

}  // namespace kgb

// the two-pass kernels, instantiated for FP32 storage only (FP64 takes the global sweep)
#define KGB_SPLIT_INSTANTIATE(T, TO)                                                                   \
    namespace kgb {                                                                                    \
    template <> FwdSmemFn<T, TO> split_pass1_lookup<T, TO>(int nn, int qmax)                          \
    {                                                                                                  \
        switch (nn * 16 + qmax) {                                                                      \
        case 2 * 16 + 8: return split_pass1_kernel<T, TO, 2, 8>;                                       \
        case 3 * 16 + 8: return split_pass1_kernel<T, TO, 3, 8>;                                       \
        case 4 * 16 + 4: return split_pass1_kernel<T, TO, 4, 4>;                                       \
        case 5 * 16 + 4: return split_pass1_kernel<T, TO, 5, 4>;                                       \
        case 6 * 16 + 4: return split_pass1_kernel<T, TO, 6, 4>;                                       \
        case 7 * 16 + 4: return split_pass1_kernel<T, TO, 7, 4>;                                       \
        case 8 * 16 + 2: return split_pass1_kernel<T, TO, 8, 2>;                                       \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> FwdSmemFn<T, TO> split_pass2_lookup<T, TO>(int nn)                                    \
    {                                                                                                  \
        switch (nn) {                                                                                  \
        case 2: return split_pass2_kernel<T, TO, 2>;                                                   \
        case 3: return split_pass2_kernel<T, TO, 3>;                                                   \
        case 4: return split_pass2_kernel<T, TO, 4>;                                                   \
        case 5: return split_pass2_kernel<T, TO, 5>;                                                   \
        case 6: return split_pass2_kernel<T, TO, 6>;                                                   \
        case 7: return split_pass2_kernel<T, TO, 7>;                                                   \
        case 8: return split_pass2_kernel<T, TO, 8>;                                                   \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    }
#define KGB_SPLIT_NONE(T, TO)                                                                          \
    namespace kgb {                                                                                    \
    template <> FwdSmemFn<T, TO> split_pass1_lookup<T, TO>(int, int) { return nullptr; }              \
    template <> FwdSmemFn<T, TO> split_pass2_lookup<T, TO>(int) { return nullptr; }                   \
    }
