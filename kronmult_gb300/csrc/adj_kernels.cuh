// Adjoint kernels of the batched Kronecker matrix-vector product.
//
// Forward (per entry k, output group e = out(k)):  y_k = K_k x_k,
// K_k = kron(A_{k,0}, ..., A_{k,d-1}).  With g_e = dL/d(output e):
//   grad_input[k]  += K_k^T g_e = kron(A_{k,0}^T, ..., A_{k,d-1}^T) g_e
//   grad_A_{k,i}   += G_(i) P_(i)^T          (n x n, summed over entries sharing A)
// where p_i = (I x .. x I x A_{i+1} x .. x A_{d-1}) x_k  (modes after i applied),
//       q_i = (A_0^T x .. x A_{i-1}^T x I x .. x I) g_e  (modes before i applied),
// and G_(i), P_(i) are the mode-i unfoldings of q_i and p_i.  The reference has no
// adjoint; kronmult_batched applied with transposed factors gives grad_input
// (kronmult_omp/kronmult.hpp:77-104), which the tests use as the check.
//
// Layouts.  The p-sweep is the forward's backward sweep (contract the fastest
// index, put the result index slowest): after applying modes d-1..i+1 the index
// order (slowest..fastest) is (j_{i+1}..j_{d-1}, l_0..l_{i-1}, l_i), so
//     P_(i)[c, t] = p_i[c + n*t].
// The q-sweep contracts the SLOWEST index and puts the result index fastest:
//     Z[r + n*t] = sum_k A_i(k, r) Q[t + R*k],   R = N/n,
// so after modes 0..i-1 the order is (j_i, j_{i+1}..j_{d-1}, l_0..l_{i-1}) and
//     G_(i)[r, t] = q_i[t + R*r]
// with the same ordering of the remaining index t as P_(i).  After all d modes q
// is K^T g in natural order: the grad_input.
//
// The forward partial products p_i are recomputed in shared memory rather than
// stored in global memory: all d of them are kept when they fit, otherwise each
// one is rebuilt from x when the q-sweep reaches it.
#pragma once
#include "fwd_kernels.cuh"

namespace kgb {

template <typename T> struct AdjArgs {
    const T *const *mats;   // nb*d factor pointers
    const T *const *in;     // nb forward inputs
    const T *const *gout;   // nb output-gradient pointers (g of the output entry k adds into)
    T *const *gin;          // nb grad_input pointers (+=), or null
    T *const *gmats;        // nb*d grad-factor pointers (+=), or null
    long long nb;
    int d, n, stride, gstride;
    int N;
    int team_size, teams_per_cta, entries_per_team;
    long long balanced_teams;  // > 0: team t takes entries [t*nb/B, (t+1)*nb/B) of B teams
    int team_elems;         // elements of T per team slice
    int npad;               // padded vector length
    int store_all;          // 1: keep all d partial products; 0: rebuild each from x
    int slices;             // split of the grad contraction over the team
};

// Entries of one team: contiguous ranges of (nearly) equal length over every team
// slot of the grid, or fixed runs of entries_per_team.
template <typename T>
__device__ __forceinline__ void adj_team_range(const AdjArgs<T> &a, long long team, long long &b, long long &e)
{
    if (a.balanced_teams > 0) {
        b = team * a.nb / a.balanced_teams;
        e = (team + 1) * a.nb / a.balanced_teams;
    } else {
        b = team * a.entries_per_team;
        e = min(b + (long long)a.entries_per_team, a.nb);
    }
}

// Every phase maps threads to individual output elements (not to whole fibres), so
// that all lanes of a warp have work for any n: with n = 6 and 32-thread teams a
// fibre mapping would leave 28 of 32 lanes idle in every second pass, and the FP64
// pipe is charged per warp instruction.

// NN > 0: n known at compile time (index arithmetic and k-loops resolved, fibres read
// with their widest aligned loads); NN = 0: n = the run-time argument.

// forward-style mode product (contract the fastest index), src -> dst:
// dst[c + r*F] = sum_k A(r, k) src[k + c*n]
template <typename T, int NN>
__device__ __forceinline__ void mode_fast_elem(const T *__restrict__ src, T *__restrict__ dst, const T *M, int n_rt,
                                               int N, const Team &tm)
{
    const int n = NN ? NN : n_rt;
    const int F = N / n;
    for (int q = tm.rank; q < N; q += tm.size) {
        // row r = q % n of fibre c = q / n: lanes of one fibre read the same words
        const int c = q / n, r = q - c * n;
        const T *x = src + c * n;
        T s = T(0);
        if constexpr (NN > 0) {
            T xv[NN];
            load_fibre<T, NN>(x, xv);
#pragma unroll
            for (int k = 0; k < NN; ++k) s = fma_t<T>(M[r + k * NN], xv[k], s);
        } else {
#pragma unroll 8
            for (int k = 0; k < n; ++k) s = fma_t<T>(M[r + k * n], x[k], s);
        }
        dst[c + r * F] = s;
    }
}

// transposed mode product contracting the slowest index, in place through registers:
// Z[r + n*t] = sum_k A(k, r) Q[t + R*k]
template <typename T, int NN, int EMAX>
__device__ __forceinline__ void mode_slow_elem(T *buf, const T *M, int n_rt, int N, const Team &tm)
{
    const int n = NN ? NN : n_rt;
    const int R = N / n;
    T z[EMAX];
#pragma unroll
    for (int j = 0; j < EMAX; ++j) {
        const int p = tm.rank + j * tm.size;
        if (p < N) {
            const int t = p / n, r = p - t * n;
            T s = T(0);
#pragma unroll 8
            for (int k = 0; k < n; ++k) s = fma_t<T>(M[k + r * n], buf[t + R * k], s);
            z[j] = s;
        }
    }
    tm.sync();
#pragma unroll
    for (int j = 0; j < EMAX; ++j) {
        const int p = tm.rank + j * tm.size;
        if (p < N) buf[p] = z[j];
    }
    tm.sync();
}

// OCC: the FP64 form for teams of at most 256 threads with at most 4 outputs per thread,
// bounded to 80 registers (no spills) so that 3 CTAs of 256 threads fit an SM; the
// default form admits teams of up to 512 threads.
template <typename T, int NN, int EMAX, bool OCC = false>
__global__ void __launch_bounds__(OCC ? 256 : 512, OCC ? 3 : 1) adj_elem_kernel(const AdjArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    const int n = NN ? NN : a.n, N = a.N, d = a.d, R = N / n, P = n * n;
    T *base = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    // slice layout: [p buffers][q][fac d*P][gacc d*P][gpart slices*P][cur grad pointers d]
    const int np = a.store_all ? d : 3;
    T *pb = base;
    T *qb = pb + (size_t)np * a.npad;
    T *fac = qb + a.npad;
    T *gacc = fac + d * P;
    T *gpart = gacc + d * P;
    T **curp = reinterpret_cast<T **>(gpart + a.slices * P + ((a.slices * P) & 1));
    const bool want_gin = a.gin != nullptr;
    const bool want_gA = a.gmats != nullptr;

    const long long team_global = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    long long e, e_end;
    adj_team_range(a, team_global, e, e_end);
    if (e >= e_end) return;

    if (want_gA) {
        for (int v = tm.rank; v < d * P; v += tm.size) gacc[v] = T(0);
        for (int v = tm.rank; v < d; v += tm.size) curp[v] = nullptr;
    }
    tm.sync();

    for (; e < e_end; ++e) {
        // flush grad accumulators whose target changes with this entry
        if (want_gA) {
            for (int v = tm.rank; v < d * P; v += tm.size) {
                const int i = v / P, pr = v - i * P;
                T *gp = a.gmats[e * d + i];
                T *cp = curp[i];
                if (gp != cp) {
                    if (cp != nullptr) {
                        const int r = pr % n, c = pr / n;
                        atomic_add<T>(cp + r + (size_t)c * a.gstride, gacc[v]);
                    }
                    gacc[v] = T(0);
                }
            }
            tm.sync();
            for (int v = tm.rank; v < d; v += tm.size) curp[v] = a.gmats[e * d + v];
        }
        // stage x (as p_{d-1}), g, and the factors fac[i*P + r + k*n] = A_i(r, k)
        T *xbuf = a.store_all ? pb + (size_t)(d - 1) * a.npad : pb;
        stage_vector(xbuf, a.in[e], N, tm);
        stage_vector(qb, a.gout[e], N, tm);
        {
            const T *const *mats = a.mats + e * d;
            for (int idx = tm.rank; idx < d * P; idx += tm.size) {
                const int i = idx / P, rem = idx - i * P, k = rem / n, r = rem - k * n;
                fac[idx] = mats[i][r + (size_t)k * a.stride];
            }
        }
        tm.sync();
        if (a.store_all) {
            for (int i = d - 1; i >= 1; --i) {
                mode_fast_elem<T, NN>(pb + (size_t)i * a.npad, pb + (size_t)(i - 1) * a.npad, fac + i * P, n, N, tm);
                tm.sync();
            }
        }
        for (int i = 0; i < d; ++i) {
            if (want_gA) {
                const T *pi;
                if (a.store_all) {
                    pi = pb + (size_t)i * a.npad;
                } else {
                    // rebuild p_i = modes d-1..i+1 applied to x, ping-ponging pb[1] and pb[2]
                    const T *src = pb;
                    T *dst = pb + a.npad;
                    for (int m = d - 1; m > i; --m) {
                        mode_fast_elem<T, NN>(src, dst, fac + m * P, n, N, tm);
                        tm.sync();
                        src = dst;
                        dst = (dst == pb + a.npad) ? pb + 2 * (size_t)a.npad : pb + a.npad;
                    }
                    pi = src;
                }
                // partial G_(i) P_(i)^T over slices of t: items (pair, slice)
                const int S = a.slices;
                const int tlen = (R + S - 1) / S;
                for (int w = tm.rank; w < S * P; w += tm.size) {
                    const int pr = w % P, sl = w / P;
                    const int r = pr % n, c = pr / n;
                    const int t0 = sl * tlen, t1 = min(R, t0 + tlen);
                    T s = T(0);
                    for (int t = t0; t < t1; ++t) s = fma_t<T>(qb[t + R * r], pi[c + n * t], s);
                    gpart[w] = s;
                }
                tm.sync();
                for (int pr = tm.rank; pr < P; pr += tm.size) {
                    T s = T(0);
                    for (int sl = 0; sl < S; ++sl) s += gpart[sl * P + pr];
                    gacc[i * P + pr] += s;
                }
            }
            if (i < d - 1 || want_gin) mode_slow_elem<T, NN, EMAX>(qb, fac + i * P, n, N, tm);
        }
        if (want_gin) {
            T *gi = a.gin[e];
            for (int v = tm.rank; v < N; v += tm.size) atomic_add<T>(gi + v, qb[v]);
        }
        tm.sync();
    }
    if (want_gA) {
        tm.sync();
        for (int v = tm.rank; v < d * P; v += tm.size) {
            const int i = v / P, pr = v - i * P;
            T *cp = curp[i];
            if (cp != nullptr) {
                const int r = pr % n, c = pr / n;
                atomic_add<T>(cp + r + (size_t)c * a.gstride, gacc[v]);
            }
        }
    }
}

// ---- fibre-mapped variant (compile-time n): each thread owns whole fibres and keeps
// them in registers; used for FP32, where register reuse matters more than idle lanes

// forward-style mode product (contract fastest index), src -> dst (distinct buffers)
template <typename T, int NN, int QMAX>
__device__ __forceinline__ void mode_fast(const T *__restrict__ src, T *__restrict__ dst, const T *M, int F,
                                          const Team &tm)
{
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int c = tm.rank + q * tm.size;
        if (c < F) {
            T xv[NN];
            load_fibre<T, NN>(src + c * NN, xv);
#pragma unroll
            for (int r = 0; r < NN; ++r) {
                T s = T(0);
#pragma unroll
                for (int k = 0; k < NN; ++k) s = fma_t<T>(M[r + k * NN], xv[k], s);
                dst[c + r * F] = s;
            }
        }
    }
}

// transposed mode product contracting the slowest index, in place through registers:
// Z[r + n*t] = sum_k A(k, r) Q[t + R*k]
template <typename T, int NN, int QMAX>
__device__ __forceinline__ void mode_slow_inplace(T *buf, const T *M, int R, const Team &tm)
{
    T z[QMAX][NN];
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int t = tm.rank + q * tm.size;
        if (t < R) {
            T qv[NN];
#pragma unroll
            for (int k = 0; k < NN; ++k) qv[k] = buf[t + R * k];
#pragma unroll
            for (int r = 0; r < NN; ++r) {
                T s = T(0);
#pragma unroll
                for (int k = 0; k < NN; ++k) s = fma_t<T>(M[k + r * NN], qv[k], s);
                z[q][r] = s;
            }
        }
    }
    tm.sync();
#pragma unroll
    for (int q = 0; q < QMAX; ++q) {
        const int t = tm.rank + q * tm.size;
        if (t < R) {
#pragma unroll
            for (int r = 0; r < NN; ++r) buf[r + NN * t] = z[q][r];
        }
    }
    tm.sync();
}

// teams of at most 256 threads; 80 registers, 3 CTAs per SM
template <typename T, int NN, int QMAX>
__global__ void __launch_bounds__(256, 3) adj_smem_kernel(const AdjArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Team tm(a.team_size);
    constexpr int P = NN * NN;
    const int N = a.N, d = a.d, R = N / NN;
    T *base = reinterpret_cast<T *>(smem_raw) + (size_t)tm.id * a.team_elems;
    // slice layout: [p buffers][q][fac d*P][gacc d*P][gpart slices*P][cur grad pointers d]
    const int np = a.store_all ? d : 3;
    T *pb = base;
    T *qb = pb + (size_t)np * a.npad;
    T *fac = qb + a.npad;
    T *gacc = fac + d * P;
    T *gpart = gacc + d * P;
    T **curp = reinterpret_cast<T **>(gpart + a.slices * P + ((a.slices * P) & 1));
    const bool want_gin = a.gin != nullptr;
    const bool want_gA = a.gmats != nullptr;

    const long long team_global = (long long)blockIdx.x * a.teams_per_cta + tm.id;
    long long e, e_end;
    adj_team_range(a, team_global, e, e_end);
    if (e >= e_end) return;

    if (want_gA) {
        for (int v = tm.rank; v < d * P; v += tm.size) gacc[v] = T(0);
        for (int v = tm.rank; v < d; v += tm.size) curp[v] = nullptr;
    }
    tm.sync();

    for (; e < e_end; ++e) {
        // flush grad accumulators whose target changes with this entry
        if (want_gA) {
            for (int v = tm.rank; v < d * P; v += tm.size) {
                const int i = v / P, pr = v - i * P;
                T *gp = a.gmats[e * d + i];
                T *cp = curp[i];
                if (gp != cp) {
                    if (cp != nullptr) {
                        const int r = pr % NN, c = pr / NN;
                        atomic_add<T>(cp + r + (size_t)c * a.gstride, gacc[v]);
                    }
                    gacc[v] = T(0);
                }
            }
            tm.sync();
            for (int v = tm.rank; v < d; v += tm.size) curp[v] = a.gmats[e * d + v];
        }
        // stage x (as p_{d-1}), g, and the factors
        T *xbuf = a.store_all ? pb + (size_t)(d - 1) * a.npad : pb;
        stage_vector(xbuf, a.in[e], N, tm);
        stage_vector(qb, a.gout[e], N, tm);
        stage_factors<T, NN>(fac, a.mats + e * d, d, a.stride, tm);
        tm.sync();
        if (a.store_all) {
            for (int i = d - 1; i >= 1; --i) {
                mode_fast<T, NN, QMAX>(pb + (size_t)i * a.npad, pb + (size_t)(i - 1) * a.npad, fac + i * P, R, tm);
                tm.sync();
            }
        }
        for (int i = 0; i < d; ++i) {
            if (want_gA) {
                const T *pi;
                if (a.store_all) {
                    pi = pb + (size_t)i * a.npad;
                } else {
                    // rebuild p_i = modes d-1..i+1 applied to x, ping-ponging pb[1] and pb[2]
                    const T *src = pb;
                    T *dst = pb + a.npad;
                    for (int m = d - 1; m > i; --m) {
                        mode_fast<T, NN, QMAX>(src, dst, fac + m * P, R, tm);
                        tm.sync();
                        src = dst;
                        dst = (dst == pb + a.npad) ? pb + 2 * (size_t)a.npad : pb + a.npad;
                    }
                    pi = src;
                }
                // partial G_(i) P_(i)^T over slices of t: items (row r, slice); an item
                // reads G(r, t) once and the whole fibre P(:, t) with vector loads and
                // keeps a row of NN sums in registers
                const int S = a.slices;
                const int tlen = (R + S - 1) / S;
                for (int w = tm.rank; w < S * NN; w += tm.size) {
                    const int r = w % NN, sl = w / NN;
                    const int t0 = sl * tlen, t1 = min(R, t0 + tlen);
                    T s[NN];
#pragma unroll
                    for (int c = 0; c < NN; ++c) s[c] = T(0);
                    for (int t = t0; t < t1; ++t) {
                        const T gv = qb[t + R * r];
                        T pv[NN];
                        load_fibre<T, NN>(pi + NN * t, pv);
#pragma unroll
                        for (int c = 0; c < NN; ++c) s[c] = fma_t<T>(gv, pv[c], s[c]);
                    }
#pragma unroll
                    for (int c = 0; c < NN; ++c) gpart[sl * P + r + NN * c] = s[c];
                }
                tm.sync();
                for (int pr = tm.rank; pr < P; pr += tm.size) {
                    T s = T(0);
                    for (int sl = 0; sl < S; ++sl) s += gpart[sl * P + pr];
                    gacc[i * P + pr] += s;
                }
            }
            if (i < d - 1 || want_gin) mode_slow_inplace<T, NN, QMAX>(qb, fac + i * P, R, tm);
        }
        if (want_gin) {
            T *gi = a.gin[e];
            for (int v = tm.rank; v < N; v += tm.size) atomic_add<T>(gi + v, qb[v]);
        }
        tm.sync();
    }
    if (want_gA) {
        tm.sync();
        for (int v = tm.rank; v < d * P; v += tm.size) {
            const int i = v / P, pr = v - i * P;
            T *cp = curp[i];
            if (cp != nullptr) {
                const int r = pr % NN, c = pr / NN;
                atomic_add<T>(cp + r + (size_t)c * a.gstride, gacc[v]);
            }
        }
    }
}

template <typename T> using AdjFn = void (*)(const AdjArgs<T>);
template <typename T> AdjFn<T> adj_lookup(int nn, int emax);
// the 3-CTA form (OCC) for compile-time n = 2..8 and EMAX <= 4; null otherwise
template <typename T> AdjFn<T> adj_occ_lookup(int nn, int emax);
template <typename T> AdjFn<T> adj_fibre_lookup(int nn, int qmax);

}  // namespace kgb

// element-mapped kernels of one n (0 = run-time n), lookup key n * 32 + EMAX
#define KGB_ADJ_ELEM_CASES(T, NN)                                                                      \
    case NN * 32 + 1: return adj_elem_kernel<T, NN, 1>;                                                \
    case NN * 32 + 2: return adj_elem_kernel<T, NN, 2>;                                                \
    case NN * 32 + 4: return adj_elem_kernel<T, NN, 4>;                                                \
    case NN * 32 + 8: return adj_elem_kernel<T, NN, 8>;                                                \
    case NN * 32 + 16: return adj_elem_kernel<T, NN, 16>;

#define KGB_ADJ_OCC_CASES(T, NN)                                                                       \
    case NN * 32 + 1: return adj_elem_kernel<T, NN, 1, true>;                                          \
    case NN * 32 + 2: return adj_elem_kernel<T, NN, 2, true>;                                          \
    case NN * 32 + 4: return adj_elem_kernel<T, NN, 4, true>;

// run-time n only (nn is ignored)
#define KGB_ADJ_INSTANTIATE(T)                                                                         \
    namespace kgb {                                                                                    \
    template <> AdjFn<T> adj_lookup<T>(int, int emax)                                                  \
    {                                                                                                  \
        switch (emax) {                                                                                \
            KGB_ADJ_ELEM_CASES(T, 0)                                                                   \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> AdjFn<T> adj_occ_lookup<T>(int, int) { return nullptr; }                               \
    }

// compile-time n for 2 <= n <= 8, run-time n otherwise
#define KGB_ADJ_INSTANTIATE_NN(T)                                                                      \
    namespace kgb {                                                                                    \
    template <> AdjFn<T> adj_lookup<T>(int nn, int emax)                                               \
    {                                                                                                  \
        switch ((nn >= 2 && nn <= 8 ? nn : 0) * 32 + emax) {                                           \
            KGB_ADJ_ELEM_CASES(T, 0)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 2)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 3)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 4)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 5)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 6)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 7)                                                                   \
            KGB_ADJ_ELEM_CASES(T, 8)                                                                   \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    template <> AdjFn<T> adj_occ_lookup<T>(int nn, int emax)                                           \
    {                                                                                                  \
        switch (nn * 32 + emax) {                                                                      \
            KGB_ADJ_OCC_CASES(T, 2)                                                                    \
            KGB_ADJ_OCC_CASES(T, 3)                                                                    \
            KGB_ADJ_OCC_CASES(T, 4)                                                                    \
            KGB_ADJ_OCC_CASES(T, 5)                                                                    \
            KGB_ADJ_OCC_CASES(T, 6)                                                                    \
            KGB_ADJ_OCC_CASES(T, 7)                                                                    \
            KGB_ADJ_OCC_CASES(T, 8)                                                                    \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    }

// fibre-mapped adjoint instantiations (used for FP32)
#define KGB_ADJ_FIBRE_INSTANTIATE(T)                                                                   \
    namespace kgb {                                                                                    \
    template <> AdjFn<T> adj_fibre_lookup<T>(int nn, int qmax)                                         \
    {                                                                                                  \
        switch (nn * 16 + qmax) {                                                                      \
        case 2 * 16 + 1: return adj_smem_kernel<T, 2, 1>;                                              \
        case 2 * 16 + 2: return adj_smem_kernel<T, 2, 2>;                                              \
        case 2 * 16 + 4: return adj_smem_kernel<T, 2, 4>;                                              \
        case 3 * 16 + 1: return adj_smem_kernel<T, 3, 1>;                                              \
        case 3 * 16 + 2: return adj_smem_kernel<T, 3, 2>;                                              \
        case 3 * 16 + 4: return adj_smem_kernel<T, 3, 4>;                                              \
        case 4 * 16 + 1: return adj_smem_kernel<T, 4, 1>;                                              \
        case 4 * 16 + 2: return adj_smem_kernel<T, 4, 2>;                                              \
        case 4 * 16 + 4: return adj_smem_kernel<T, 4, 4>;                                              \
        case 5 * 16 + 1: return adj_smem_kernel<T, 5, 1>;                                              \
        case 5 * 16 + 2: return adj_smem_kernel<T, 5, 2>;                                              \
        case 5 * 16 + 4: return adj_smem_kernel<T, 5, 4>;                                              \
        case 6 * 16 + 1: return adj_smem_kernel<T, 6, 1>;                                              \
        case 6 * 16 + 2: return adj_smem_kernel<T, 6, 2>;                                              \
        case 6 * 16 + 4: return adj_smem_kernel<T, 6, 4>;                                              \
        case 7 * 16 + 1: return adj_smem_kernel<T, 7, 1>;                                              \
        case 7 * 16 + 2: return adj_smem_kernel<T, 7, 2>;                                              \
        case 7 * 16 + 4: return adj_smem_kernel<T, 7, 4>;                                              \
        case 8 * 16 + 1: return adj_smem_kernel<T, 8, 1>;                                              \
        case 8 * 16 + 2: return adj_smem_kernel<T, 8, 2>;                                              \
        case 8 * 16 + 4: return adj_smem_kernel<T, 8, 4>;                                              \
        default: return nullptr;                                                                       \
        }                                                                                              \
    }                                                                                                  \
    }
