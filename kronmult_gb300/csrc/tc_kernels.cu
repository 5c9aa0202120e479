// Tensor-core (tcgen05) forward for n = 8: FP32 storage, TF32 or BF16 mode
// products with FP32 accumulation in tensor memory, FP64 output accumulation.
//
// For n = 8 every mode product of the backward sweep (kronmult_gpu/kronmult.cu:54-78)
//     Y[c + r*F] = sum_k A_i(r, k) X[k + 8c],   F = N/8 fibres
// is a dense GEMM D[c][r] = sum_k X^T[c][k] A_i^T[k][r] with M = F, N = 8, K = 8.
// It runs as tcgen05.mma.cta_group::1 with M = 128 fibres per instruction
// (N = 16, the smallest N for M = 128; K = 8 for TF32, K = 16 for BF16 with the
// upper 8 zero).  Operands live in shared memory in the canonical K-major,
// no-swizzle layout of 8-row x 16-byte core matrices; the accumulator lives in
// tensor memory, one 16-column block per PAIR of 128-fibre tiles: the even tile
// multiplies B = [A_i^T | 0] into columns 0..7, the odd tile B = [0 | A_i^T]
// accumulated into columns 8..15, so no accumulator column is padding and a CTA
// needs half the columns (more CTAs per SM).  After each mode the four warps read
// their 32 TMEM lanes (tcgen05.ld.32x32b), round to the operand type and write
// the mode output straight into the next mode's operand layout at the rotated
// positions, so the vector never leaves shared memory.
//
// BF16 (fwd_tc_bf16_kernel) keeps the vector operand MN-major (8 consecutive fibres =
// 16 contiguous bytes per K row of a core matrix) and applies the modes in the order
// 0, 1, ..., d-1: the contracted index is then always the most significant digit of the
// fibre index, and the 8 outputs a thread reads from its TMEM lane (one fibre, the 8
// values of the new index) are 8 consecutive fibres of the next mode's operand, written
// with ONE 16-byte store.  The first operand is the natural vector itself read as
// MN-major (fibre = the fastest d-1 indices, K = the slowest), converted 8 values per
// 16-byte store.  Two 128-fibre tiles share one MMA: K = 16 holds the even tile in K
// rows 0..7 and the odd one in rows 8..15, against the block-diagonal factor operand
// [A_i 0; 0 A_i], so the operand carries no zero padding.  TF32 (fwd_tc_kernel; K = 8
// per MMA) keeps the backward order and the K-major operand, written element by element.
//
// One CTA = one warpgroup (128 threads) works on one entry at a time; several
// CTAs per SM overlap the input loads.  Consecutive entries with the same
// output pointer are summed in tensor memory and added with FP64 atomics.
//
// Every wait on an mbarrier is bounded; on timeout the kernel records an error
// code in a device word (kronmult_device_error) and leaves after freeing its
// tensor memory.
#include <cuda_bf16.h>
#include <cstdint>
#include "fwd_launch.cuh"

namespace kgb {

__device__ unsigned int g_tc_error = 0;  // 0 = ok; otherwise the code of the first failure

namespace {

constexpr int kTcThreads = 128;
constexpr int kTileRows = 128;               // fibres per MMA (M)
constexpr int kTileBytes = kTileRows * 32;   // one K-major tile: 128 rows x 32 bytes
constexpr int kBBytes = 16 * 32;             // one factor operand: 16 rows x 32 bytes
constexpr unsigned kWaitLimit = 1u << 22;    // bounded mbarrier polling
// BF16 MN-major vector operand: per group of 8 fibres, K rows 0..7 (128 bytes), K rows
// 8..15 (128 bytes), then 16 bytes of padding, so that 8 consecutive groups start in 8
// different 16-byte bank slots
constexpr uint32_t kMnLbo = 128;                 // K-group stride
constexpr uint32_t kMnSbo = 272;                 // 8-fibre group stride

enum : int { KIND_TF32 = 0, KIND_BF16 = 1 };

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) of a 32-byte-row K-major operand in core-matrix layout:
// core matrix = 8 rows x 16 bytes (128 B contiguous); K-adjacent core matrices are
// 128 B apart (leading byte offset), M-adjacent 8-row groups 256 B apart (stride byte offset)
__device__ __forceinline__ uint32_t core_offset(uint32_t row, uint32_t kbyte)
{
    return (row >> 3) * 256u + (kbyte >> 4) * 128u + (row & 7u) * 16u + (kbyte & 15u);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo = 128u, uint32_t sbo = 256u)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);          // start address
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;      // leading byte offset (K direction)
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;      // stride byte offset (M/N direction)
    d |= (uint64_t)1u << 46;                          // descriptor version for sm_100 family
    return d;                                         // base offset 0, no swizzle
}

// The A operand (the vector: `tiles` tiles of 128 rows) uses the same core matrices
// with a different arrangement: the k-chunk-0 core matrices of all rows first (8-row
// groups 128 B apart, SBO = 128), the k-chunk-1 ones LBO = tiles*2048 + 64 bytes
// later.  The two 16-byte halves of a row then sit 64 bytes apart modulo the 128-byte
// bank row, so the epilogue's stores (consecutive lanes = consecutive rows, both
// halves) and the staging conversion hit distinct banks.
__device__ __forceinline__ uint32_t a_lbo(int tiles) { return (uint32_t)tiles * 2048u + 64u; }
__device__ __forceinline__ uint32_t a_offset(uint32_t row, uint32_t kbyte, uint32_t lbo)
{
    return (row >> 3) * 128u + (kbyte >> 4) * lbo + (row & 7u) * 16u + (kbyte & 15u);
}

template <int KIND, bool A_MN_MAJOR = false> __device__ __forceinline__ constexpr uint32_t instr_desc()
{
    // D = F32; A, B = TF32 (2) or BF16 (1); A K-major, or MN-major (bit 15, "transpose A");
    // B K-major; N = 16; M = 128
    return (1u << 4) | ((KIND == KIND_TF32 ? 2u : 1u) << 7) | ((KIND == KIND_TF32 ? 2u : 1u) << 10) |
           ((A_MN_MAJOR ? 1u : 0u) << 15) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    if constexpr (KIND == KIND_TF32) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
            "l"(adesc), "l"(bdesc), "r"(instr_desc<KIND>()), "r"(accumulate));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
            "l"(adesc), "l"(bdesc), "r"(instr_desc<KIND>()), "r"(accumulate));
    }
}

// BF16 MMA with an MN-major A operand (the vector) and a K-major B operand (the factor)
__device__ __forceinline__ void mma_bf16_mn(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(instr_desc<KIND_BF16, true>()), "r"(accumulate));
}

// 8 FP32 values rounded to BF16 (nearest even), packed in order into 16 bytes
__device__ __forceinline__ uint4 pack_bf16x8(float a0, float a1, float a2, float a3, float a4, float a5, float a6,
                                             float a7)
{
    uint4 r;
    __nv_bfloat162 h;
    h = __floats2bfloat162_rn(a0, a1);
    r.x = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2bfloat162_rn(a2, a3);
    r.y = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2bfloat162_rn(a4, a5);
    r.z = *reinterpret_cast<uint32_t *>(&h);
    h = __floats2bfloat162_rn(a6, a7);
    r.w = *reinterpret_cast<uint32_t *>(&h);
    return r;
}

// BF16 K-stacked operand: the tiles of a pair (128 fibres each) share 8-fibre groups; K
// rows 0..7 of a group hold the even tile, K rows 8..15 (one K-group = 128 bytes later)
// the odd one, so one MMA with K = 16 and a block-diagonal factor operand computes both
// tiles and no operand byte is padding.  Byte offset of fibre group g, K row kk:
constexpr uint32_t kPairBytes = 16 * kMnSbo;  // 16 groups of 8 fibres
constexpr int kBf16B = 512;                   // factor operand: 16 rows x 16 K x 2 bytes
__device__ __forceinline__ uint32_t mn_offset(uint32_t g, uint32_t kk)
{
    const uint32_t t = g >> 4;  // tile of the group
    return (t >> 1) * kPairBytes + (g & 15u) * kMnSbo + (t & 1u) * kMnLbo + kk * 16u;
}

// FP64 addition into global memory without a returned value
__device__ __forceinline__ void red_add_f64(double *p, double v)
{
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

// 8x8 transpose across the 8 lanes of each aligned lane octet: afterwards lane l's v[j]
// is lane j's former v[l] (three butterfly stages of register-pair exchanges)
__device__ __forceinline__ void octet_transpose(float (&v)[8], int lane)
{
#pragma unroll
    for (int s = 4; s >= 1; s >>= 1) {
        const bool upper = (lane & s) != 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j & s) continue;
            const float send = upper ? v[j] : v[j | s];
            const float recv = __shfl_xor_sync(0xffffffffu, send, s);
            if (upper)
                v[j] = recv;
            else
                v[j | s] = recv;
        }
    }
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, unsigned limit = kWaitLimit)
{
    for (unsigned it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive columns of this warp's 32 lanes: the two tiles of one block
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v0)[8], float (&v1)[8])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        v0[j] = __uint_as_float(r[j]);
        v1[j] = __uint_as_float(r[8 + j]);
    }
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ float to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// 8 FP32 values split into BF16 pairs v = hi + lo: hi rounded to nearest, lo the rounded
// remainder (v - hi is exact in FP32), each set packed in order into 16 bytes
__device__ __forceinline__ void split_bf16x8(const float (&v)[8], uint4 &hi, uint4 &lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat162 hb = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        h[i] = *reinterpret_cast<const uint32_t *>(&hb);
        // hi back in FP32 (a BF16 value is the upper half of its FP32 bits), both lanes at
        // once; the remainders with one packed subtraction
        const f2 hf = ((unsigned long long)(h[i] & 0xFFFF0000u) << 32) | ((unsigned long long)(h[i] & 0xFFFFu) << 16);
        float r0, r1;
        f2_unpack(f2_sub(f2_pack(v[2 * i], v[2 * i + 1]), hf), r0, r1);
        const __nv_bfloat162 lb = __floats2bfloat162_rn(r0, r1);
        l[i] = *reinterpret_cast<const uint32_t *>(&lb);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// store one value of the operand element (row, k) in the operand type of KIND: B
// operands (factors) in the plain core-matrix layout, A (lbo != 0) in the split one
template <int KIND>
__device__ __forceinline__ void put(unsigned char *base, uint32_t row, uint32_t k, float v, uint32_t lbo = 0)
{
    constexpr uint32_t es = KIND == KIND_TF32 ? 4u : 2u;
    const uint32_t off = lbo ? a_offset(row, k * es, lbo) : core_offset(row, k * es);
    if constexpr (KIND == KIND_TF32) {
        *reinterpret_cast<float *>(base + off) = to_tf32(v);
    } else {
        *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
    }
}

}  // namespace

struct TcArgs {
    const float *const *mats;
    const float *const *in;
    double *const *out;
    long long nb;
    int d, stride, N, tiles, tmem_cols, entries_per_cta;
};

// per-thread pointers of one entry, loaded one entry ahead of the copies that use them
constexpr int kTcFacSlots = 2;  // factor elements per thread: d*64 <= 256 = 2 x 128 threads
struct TcPtrs {
    const float *src;
    const float *mat[kTcFacSlots];
};

__device__ __forceinline__ void tc_load_ptrs(TcPtrs &p, const TcArgs &a, long long e, int tid)
{
    p.src = a.in[e];
#pragma unroll
    for (int s = 0; s < kTcFacSlots; ++s) {
        const int idx = tid + s * kTcThreads;
        p.mat[s] = idx < a.d * 64 ? a.mats[e * a.d + (idx >> 6)] : nullptr;
    }
}

// asynchronous copy of one entry's vector into the raw staging slot (natural order)
// and of its factor elements into registers: thread tid holds fv[s] = A_i(r, k) for
// idx = tid + 128 s, i = idx / 64, r = idx % 8, k = (idx / 8) % 8.  The vector is one TMA
// bulk copy (cp.async.bulk) issued by thread 0 and completed on the staging barrier
// `sbar` when its source is 16-byte aligned; otherwise every thread copies 4-byte
// elements with cp.async and thread 0 completes the barrier's phase without bytes.
// Either way the staging barrier completes exactly one phase per entry.  The factor
// loads are plain loads consumed one entry later, so their latency is hidden too.
__device__ __forceinline__ void tc_stage_async(float *raw, float (&fv)[kTcFacSlots], const TcPtrs &p,
                                               const TcArgs &a, int tid, uint32_t sbar)
{
    const int N = a.N;
    const unsigned bytes = (unsigned)N * 4u;
    if (((reinterpret_cast<uintptr_t>(p.src) & 15u) == 0) && ((bytes & 15u) == 0)) {
        if (tid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(raw)),
                "l"(p.src), "r"(bytes), "r"(sbar)
                : "memory");
        }
    } else {
        for (int q = tid; q < N; q += kTcThreads) cp_async<4>(raw + q, p.src + q);
        if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sbar) : "memory");
    }
    cp_async_commit();
#pragma unroll
    for (int s = 0; s < kTcFacSlots; ++s) {
        const int idx = tid + s * kTcThreads;
        if (idx < a.d * 64) {
            const int r = idx & 7, k = (idx >> 3) & 7;
            fv[s] = __ldg(p.mat[s] + r + (size_t)k * a.stride);
        }
    }
}

template <int KIND> __global__ void __launch_bounds__(kTcThreads, 6) fwd_tc_kernel(const TcArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = a.N, F = N / 8, d = a.d;
    // shared memory: one raw staging slot for the vector, operand A, operands B, barriers.
    // The slot is refilled with the next entry as soon as this entry's operands are built.
    float *raw = reinterpret_cast<float *>(smem_raw);
    unsigned char *xs = reinterpret_cast<unsigned char *>(raw + N);  // tiles x 4 KB
    unsigned char *bs = xs + (size_t)a.tiles * kTileBytes + 64;            // d x 512 B: [A_i^T | 0]
    unsigned char *bs2 = bs + (size_t)d * kBBytes;                         // d x 512 B: [0 | A_i^T]
    uint64_t *mbar = reinterpret_cast<uint64_t *>(bs2 + (size_t)d * kBBytes);  // MMA completion
    uint64_t *sbar = mbar + 1;                                                  // staging completion
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    long long e = (long long)blockIdx.x * a.entries_per_cta;
    const long long e_end = min(e + (long long)a.entries_per_cta, a.nb);
    if (e >= e_end) return;

    // operands zeroed once: the zero half of each B (rows 8..15 of [A^T | 0], rows 0..7 of
    // [0 | A^T]) and, for BF16, the K 8..15 half of A stay zero
    for (int v = tid; v < (a.tiles * kTileBytes + 64 + 2 * d * kBBytes) / 16; v += kTcThreads)
        reinterpret_cast<int4 *>(xs)[v] = make_int4(0, 0, 0, 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    const uint32_t sbar_a = smem_u32(sbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    TcPtrs nxt;
    float fv[kTcFacSlots] = {0.f, 0.f};  // factor elements of the entry staged last
    tc_load_ptrs(nxt, a, e, tid);
    tc_stage_async(raw, fv, nxt, a, tid, sbar_a);
    if (e + 1 < e_end) tc_load_ptrs(nxt, a, e + 1, tid);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int blocks = (a.tiles + 1) / 2;        // 16-column accumulator blocks, two tiles each
    const uint32_t tacc = tmem + 16u * blocks;   // run accumulator after the mode output
    const uint32_t mbar_a = smem_u32(mbar);
    const uint32_t xs_a = smem_u32(xs), bs_a = smem_u32(bs), bs2_a = smem_u32(bs2);
    const uint32_t lboa = a_lbo(a.tiles);  // A operand: k-chunk-1 core matrices this far after chunk 0
    uint32_t phase = 0, sphase = 0;
    bool failed = false;
    bool staging = true;  // a staging copy is in flight whose phase has not been waited for
    double *cur = nullptr;
    constexpr int MAXT = 4;  // tiles per entry (N <= 4096)

    // run sum (TMEM accumulator) -> FP64 atomics into `dst`
    auto flush = [&](double *dst) {
        auto add_tile = [&](int t, const float (&v)[8]) {
            const int c = t * kTileRows + warp * 32 + lane;
            if (t < a.tiles && c < F)
#pragma unroll
                for (int r = 0; r < 8; ++r) red_add_f64(dst + c + r * F, (double)v[r]);
        };
#pragma unroll
        for (int j = 0; j < MAXT / 2; ++j) {
            if (j < blocks) {
                float v0[8], v1[8];
                tmem_ld16(tacc + ((uint32_t)(warp * 32) << 16) + 16u * j, v0, v1);
                tmem_wait_ld();
                add_tile(2 * j, v0);
                add_tile(2 * j + 1, v1);
            }
        }
    };

    for (; e < e_end; ++e) {
        double *o = a.out[e];
        cp_async_wait_all();
        const bool staged = mbar_wait(sbar_a, sphase);  // the slot's bulk copy (or its empty phase)
        if (__syncthreads_or(!staged)) {  // slot complete for every thread; previous MMAs done
            if (tid == 0) atomicCAS(&g_tc_error, 0u, 1u);
            failed = true;
            break;
        }
        sphase ^= 1u;
        staging = false;
        // operands: B_i[row r][k] = A_i(r, k) (and row r + 8 of the second copy); input
        // natural index p = k + 8c -> A row c, column k
#pragma unroll
        for (int s = 0; s < kTcFacSlots; ++s) {
            const int v = tid + s * kTcThreads;
            if (v < d * 64) {
                const int i = v >> 6, r = v & 7, k = (v >> 3) & 7;
                put<KIND>(bs + (size_t)i * kBBytes, r, k, fv[s]);
                put<KIND>(bs2 + (size_t)i * kBBytes, r + 8, k, fv[s]);
            }
        }
        // natural position p = k + 8c -> operand row c, column k: the 4 values of a float4
        // are one 16-byte half of a core-matrix row
        for (int q = tid; q < N / 4; q += kTcThreads) {
            const float4 v4 = *reinterpret_cast<const float4 *>(raw + 4 * q);
            const uint32_t c = q >> 1, kbyte = (q & 1) * 16;
            *reinterpret_cast<float4 *>(xs + a_offset(c, kbyte, lboa)) =
                make_float4(to_tf32(v4.x), to_tf32(v4.y), to_tf32(v4.z), to_tf32(v4.w));
        }
        // the run continues when this entry adds into the same output as the previous one;
        // otherwise the previous run's sum leaves TMEM before the last mode overwrites it
        const bool cont = (o == cur);
        if (!cont && cur != nullptr) flush(cur);
        cur = o;
        fence_async_smem();  // the staging slot has been read (generic proxy) before the bulk copy refills it
        tc_fence_before();
        __syncthreads();
        if (e + 1 < e_end) {
            tc_stage_async(raw, fv, nxt, a, tid, sbar_a);
            staging = true;
            if (e + 2 < e_end) tc_load_ptrs(nxt, a, e + 2, tid);
        }

        for (int i = d - 1; i >= 0; --i) {
            if (tid == 0) {
                tc_fence_after();
                const uint32_t dst = i > 0 ? tmem : tacc;
                const uint32_t accumulate = (i == 0 && cont) ? 1u : 0u;
                // even tile: columns 0..7 of its block (overwriting, or adding to the run);
                // odd tile: columns 8..15, always added (the even tile's B zeroed them)
                for (int t = 0; t < a.tiles; ++t)
                    mma<KIND>(dst + 16u * (uint32_t)(t >> 1), smem_desc(xs_a + t * 2048u, lboa, 128u),
                              smem_desc(((t & 1) ? bs2_a : bs_a) + i * kBBytes), (t & 1) ? 1u : accumulate);
                mma_commit(mbar_a);
            }
            const bool ok = mbar_wait(mbar_a, phase);
            // the decision to leave must be uniform: the TMEM loads below are warp-collective
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicCAS(&g_tc_error, 0u, 1u);
                failed = true;
                break;
            }
            phase ^= 1u;
            tc_fence_after();
            if (i > 0) {
                // mode output element (row c, r) goes to natural position p = c + r*F,
                // which is operand row p/8, column p%8 of the next mode; one block (two
                // tiles) at a time keeps 16 values per thread live
                auto store_tile = [&](int t, const float (&v)[8]) {
                    const int c = t * kTileRows + warp * 32 + lane;
                    if (t < a.tiles && c < F) {
                        if (F >= 64) {
                            // F/8 a multiple of 8: row p/8 = c/8 + r*F/8 keeps its position in
                            // the 8-row group and moves r*F/64 groups, 2F bytes per r
                            const uint32_t base = a_offset((uint32_t)c >> 3, 4u * ((uint32_t)c & 7u), lboa);
#pragma unroll
                            for (int r = 0; r < 8; ++r)
                                *reinterpret_cast<float *>(xs + base + (uint32_t)r * 2u * (uint32_t)F) = to_tf32(v[r]);
                        } else {
#pragma unroll
                            for (int r = 0; r < 8; ++r) {
                                const uint32_t p = c + r * F;
                                put<KIND>(xs, p >> 3, p & 7, v[r], lboa);
                            }
                        }
                    }
                };
#pragma unroll
                for (int j = 0; j < MAXT / 2; ++j) {
                    if (j < blocks) {
                        float v0[8], v1[8];
                        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + 16u * j, v0, v1);
                        tmem_wait_ld();
                        store_tile(2 * j, v0);
                        store_tile(2 * j + 1, v1);
                    }
                }
                fence_async_smem();
                tc_fence_before();
                __syncthreads();
            }
        }
        if (failed) break;
    }
    cp_async_wait_all();
    // leaving early with a bulk copy still in flight: one more bounded wait for it, so
    // that it does not land in shared memory after this CTA is gone
    if (failed && staging) mbar_wait(sbar_a, sphase);
    if (cur != nullptr && !failed) flush(cur);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// BF16 forward (layout and mode order in the file comment).  Same pipeline as
// fwd_tc_kernel: one staging slot refilled by a bulk copy while the current entry's
// modes run, factors one entry ahead in registers, runs of entries with one output
// summed in TMEM, bounded mbarrier waits.
// SPLIT (KRONMULT_COMPUTE_BF16X3): every operand value v is held as two BF16 values,
// hi = bf16(v) and lo = bf16(v - hi), and each tile pair runs three MMAs into one FP32
// accumulator, x_hi.A_hi + x_lo.A_hi + x_hi.A_lo (the lo.lo term, 2^-16 relative, is
// dropped): about 16 significand bits per product instead of 8.  The hi and lo vector
// operands and factor operands sit side by side in the same layouts.
template <bool SPLIT>
__global__ void __launch_bounds__(kTcThreads, SPLIT ? 5 : 8) fwd_tc_bf16_kernel(const TcArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = a.N, F = N / 8, d = a.d;
    const int pairs = (a.tiles + 1) / 2;
    constexpr int kParts = SPLIT ? 2 : 1;
    float *raw = reinterpret_cast<float *>(smem_raw);                          // staging slot, N floats
    unsigned char *xs = reinterpret_cast<unsigned char *>(raw + N);           // pairs x kPairBytes (hi)
    unsigned char *xl = xs + (size_t)pairs * kPairBytes;                      // the lo parts (SPLIT)
    unsigned char *bs = xs + (size_t)kParts * pairs * kPairBytes + 64;        // d x [A_i 0; 0 A_i] (hi)
    unsigned char *bl = bs + (size_t)d * kBf16B;                              // the lo parts (SPLIT)
    uint64_t *mbar = reinterpret_cast<uint64_t *>(bs + (size_t)kParts * d * kBf16B);  // MMA completion
    uint64_t *sbar = mbar + 1;                                                // staging completion
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    long long e = (long long)blockIdx.x * a.entries_per_cta;
    const long long e_end = min(e + (long long)a.entries_per_cta, a.nb);
    if (e >= e_end) return;

    // operands zeroed once: fibres beyond F, the odd K half of an unpaired tile and the
    // off-diagonal blocks of the factor operands stay zero
    for (int v = tid; v < (int)(kParts * pairs * kPairBytes + 64 + kParts * d * kBf16B) / 16; v += kTcThreads)
        reinterpret_cast<int4 *>(xs)[v] = make_int4(0, 0, 0, 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    const uint32_t sbar_a = smem_u32(sbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    TcPtrs nxt;
    float fv[kTcFacSlots] = {0.f, 0.f};  // factor elements of the entry staged last
    tc_load_ptrs(nxt, a, e, tid);
    tc_stage_async(raw, fv, nxt, a, tid, sbar_a);
    if (e + 1 < e_end) tc_load_ptrs(nxt, a, e + 1, tid);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tacc = tmem + 16u * pairs;  // run accumulator after the mode output
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const uint32_t mbar_a = smem_u32(mbar);
    const uint32_t xs_a = smem_u32(xs), bs_a = smem_u32(bs), xl_a = smem_u32(xl), bl_a = smem_u32(bl);
    uint32_t phase = 0, sphase = 0;
    bool failed = false;
    bool staging = true;  // a staging copy is in flight whose phase has not been waited for
    double *cur = nullptr;
    constexpr int MAXP = 2;  // tile pairs per entry (N <= 4096)

    // run sum (TMEM accumulator) -> FP64 reductions into `dst`.  Fibre c of the last mode
    // holds output positions 8c + r; after an octet transpose lane l of octet o holds
    // positions 64o + 8j + l (o = c / 8), so every reduction instruction of a warp covers
    // 4 runs of 8 consecutive doubles.
    auto flush = [&](double *dst) {
        if (F < 8) {  // d = 1: one fibre, its 8 values are the whole output vector
            if (warp == 0) {
                float v0[8], v1[8];
                tmem_ld16(tacc, v0, v1);  // warp-collective: the whole warp loads
                tmem_wait_ld();
                if (lane == 0)
#pragma unroll
                    for (int r = 0; r < 8; ++r) red_add_f64(dst + r, (double)v0[r]);
            }
            return;
        }
#pragma unroll
        for (int j = 0; j < MAXP; ++j) {
            if (j < pairs) {
                float v0[8], v1[8];
                tmem_ld16(tacc + lane_base + 16u * j, v0, v1);
                tmem_wait_ld();
                octet_transpose(v0, lane);
                octet_transpose(v1, lane);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int t = 2 * j + h;
                    const int c0 = t * kTileRows + warp * 32 + (lane & ~7);  // first fibre of the octet
                    if (t < a.tiles && c0 < F) {
                        double *p = dst + 8 * c0 + (lane & 7);
#pragma unroll
                        for (int r = 0; r < 8; ++r) red_add_f64(p + 8 * r, (double)(h ? v1[r] : v0[r]));
                    }
                }
            }
        }
    };

    for (; e < e_end; ++e) {
        double *o = a.out[e];
        cp_async_wait_all();
        const bool staged = mbar_wait(sbar_a, sphase);  // the slot's bulk copy (or its empty phase)
        if (__syncthreads_or(!staged)) {  // slot complete for every thread; previous MMAs done
            if (tid == 0) atomicCAS(&g_tc_error, 0u, 1u);
            failed = true;
            break;
        }
        sphase ^= 1u;
        staging = false;
        // factor operands: B_i[n][k] = A_i(n, k) in the upper-left and lower-right blocks
#pragma unroll
        for (int s = 0; s < kTcFacSlots; ++s) {
            const int v = tid + s * kTcThreads;
            if (v < d * 64) {
                const int i = v >> 6, r = v & 7, k = (v >> 3) & 7;
                put<KIND_BF16>(bs + (size_t)i * kBf16B, r, k, fv[s]);
                put<KIND_BF16>(bs + (size_t)i * kBf16B, r + 8, k + 8, fv[s]);
                if constexpr (SPLIT) {
                    const float rem = fv[s] - __bfloat162float(__float2bfloat16_rn(fv[s]));
                    put<KIND_BF16>(bl + (size_t)i * kBf16B, r, k, rem);
                    put<KIND_BF16>(bl + (size_t)i * kBf16B, r + 8, k + 8, rem);
                }
            }
        }
        // vector operand: natural position p = fibre + F*K (K = the slowest index, mode 0,
        // contracted first), so 8 consecutive positions are 8 consecutive fibres of one K row
        if (d == 1) {
            if (tid < 8) {
                const __nv_bfloat16 h = __float2bfloat16_rn(raw[tid]);
                *reinterpret_cast<__nv_bfloat16 *>(xs + tid * 16) = h;
                if constexpr (SPLIT)
                    *reinterpret_cast<__nv_bfloat16 *>(xl + tid * 16) =
                        __float2bfloat16_rn(raw[tid] - __bfloat162float(h));
            }
        } else {
            const uint32_t fsh = 3u * (uint32_t)(d - 1);
            for (int q = tid; q < N / 8; q += kTcThreads) {
                // the two 16-byte halves in an order that keeps each 8-lane phase of the
                // 16-byte loads on 8 distinct bank slots
                const int h = (q >> 2) & 1;
                const float4 first = *reinterpret_cast<const float4 *>(raw + 8 * q + 4 * h);
                const float4 second = *reinterpret_cast<const float4 *>(raw + 8 * q + 4 * (h ^ 1));
                const float4 u = h ? second : first, w = h ? first : second;
                const uint32_t p0 = 8u * (uint32_t)q;
                const uint32_t off = mn_offset((p0 & (uint32_t)(F - 1)) >> 3, p0 >> fsh);
                if constexpr (SPLIT) {
                    const float v8[8] = {u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w};
                    uint4 hi, lo;
                    split_bf16x8(v8, hi, lo);
                    *reinterpret_cast<uint4 *>(xs + off) = hi;
                    *reinterpret_cast<uint4 *>(xl + off) = lo;
                } else {
                    *reinterpret_cast<uint4 *>(xs + off) = pack_bf16x8(u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w);
                }
            }
        }
        // the run continues when this entry adds into the same output as the previous one;
        // otherwise the previous run's sum leaves TMEM before the last mode overwrites it
        const bool cont = (o == cur);
        if (!cont && cur != nullptr) flush(cur);
        cur = o;
        fence_async_smem();  // the staging slot has been read (generic proxy) before the bulk copy refills it
        tc_fence_before();
        __syncthreads();
        if (e + 1 < e_end) {
            tc_stage_async(raw, fv, nxt, a, tid, sbar_a);
            staging = true;
            if (e + 2 < e_end) tc_load_ptrs(nxt, a, e + 2, tid);
        }

        for (int i = 0; i < d; ++i) {  // modes 0, 1, ..., d-1
            const bool last = i == d - 1;
            if (tid == 0) {
                tc_fence_after();
                const uint32_t dst = last ? tacc : tmem;
                const uint32_t accumulate = (last && cont) ? 1u : 0u;
                for (int j = 0; j < pairs; ++j) {
                    mma_bf16_mn(dst + 16u * (uint32_t)j, smem_desc(xs_a + j * kPairBytes, kMnLbo, kMnSbo),
                                smem_desc(bs_a + i * kBf16B), accumulate);
                    if constexpr (SPLIT) {
                        mma_bf16_mn(dst + 16u * (uint32_t)j, smem_desc(xl_a + j * kPairBytes, kMnLbo, kMnSbo),
                                    smem_desc(bs_a + i * kBf16B), 1u);
                        mma_bf16_mn(dst + 16u * (uint32_t)j, smem_desc(xs_a + j * kPairBytes, kMnLbo, kMnSbo),
                                    smem_desc(bl_a + i * kBf16B), 1u);
                    }
                }
                mma_commit(mbar_a);
            }
            const bool ok = mbar_wait(mbar_a, phase);
            // the decision to leave must be uniform: the TMEM loads below are warp-collective
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicCAS(&g_tc_error, 0u, 1u);
                failed = true;
                break;
            }
            phase ^= 1u;
            tc_fence_after();
            if (!last) {
                // fibre c = g + F/8 * kk with kk the next mode's index (c's top digit): the 8
                // new values become the 8 consecutive fibres 8g..8g+7 of the next operand
                const uint32_t sh = 3u * (uint32_t)(d - 2);
#pragma unroll
                for (int j = 0; j < MAXP; ++j) {
                    if (j < pairs) {
                        float v0[8], v1[8];
                        tmem_ld16(tmem + lane_base + 16u * j, v0, v1);
                        tmem_wait_ld();
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int t = 2 * j + h;
                            const int c = t * kTileRows + warp * 32 + lane;
                            if (t < a.tiles && c < F) {
                                const float(&v)[8] = h ? v1 : v0;
                                const uint32_t kk = (uint32_t)c >> sh, g = (uint32_t)c & ((1u << sh) - 1u);
                                if constexpr (SPLIT) {
                                    uint4 hi, lo;
                                    split_bf16x8(v, hi, lo);
                                    *reinterpret_cast<uint4 *>(xs + mn_offset(g, kk)) = hi;
                                    *reinterpret_cast<uint4 *>(xl + mn_offset(g, kk)) = lo;
                                } else {
                                    *reinterpret_cast<uint4 *>(xs + mn_offset(g, kk)) =
                                        pack_bf16x8(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7]);
                                }
                            }
                        }
                    }
                }
                fence_async_smem();
                tc_fence_before();
                __syncthreads();
            }
        }
        if (failed) break;
    }
    cp_async_wait_all();
    // leaving early with a bulk copy still in flight: one more bounded wait for it, so
    // that it does not land in shared memory after this CTA is gone
    if (failed && staging) mbar_wait(sbar_a, sphase);
    if (cur != nullptr && !failed) flush(cur);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// Plans and enqueues the tensor-core forward.  Returns cudaErrorNotSupported for
// shapes it does not cover (n != 8, n^d > 4096), so that the caller can fall back.
int launch_tc_forward(int kind, int d, int n, const float *const *mats, int stride, const float *const *in,
                      double *const *out, long long nb, cudaStream_t st, const kronmult_tuning *tune)
{
    if (n != 8 || d < 1) return cudaErrorNotSupported;
    const long long Nl = pow_ll(n, d);
    if (Nl > 4096) return cudaErrorNotSupported;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
    const DeviceInfo &di = device_info(dev);
    TcArgs a{};
    a.mats = mats;
    a.in = in;
    a.out = out;
    a.nb = nb;
    a.d = d;
    a.stride = stride;
    a.N = (int)Nl;
    const int F = a.N / 8;
    a.tiles = (F + kTileRows - 1) / kTileRows;
    const int pairs = (a.tiles + 1) / 2;
    int cols = 32;
    while (cols < 2 * 16 * pairs) cols *= 2;  // mode output + run accumulator
    a.tmem_cols = cols;
    const bool split = kind == KRONMULT_COMPUTE_BF16X3;
    const bool bf16 = kind == KRONMULT_COMPUTE_BF16 || split;
    const size_t parts = split ? 2 : 1;
    const size_t need = (size_t)a.N * sizeof(float) +
                        (bf16 ? parts * pairs * kPairBytes + 64 + parts * d * kBf16B
                              : (size_t)a.tiles * kTileBytes + 64 + (size_t)2 * d * kBBytes) +
                        32;  // + two mbarriers and the TMEM address
    // resident CTAs per SM are limited so that their tensor-memory columns fit in 512
    // (or to tuning.ctas_per_sm when that is fewer): each CTA reserves 1/max_ctas of the
    // SM's shared memory (less the per-CTA system reservation), so at most max_ctas fit
    int max_ctas = 512 / cols;
    if (tune && tune->ctas_per_sm > 0 && tune->ctas_per_sm < max_ctas) max_ctas = tune->ctas_per_sm;
    size_t smem = (size_t)di.smem_per_sm / max_ctas - (size_t)di.smem_reserved_cta;
    smem &= ~(size_t)15;
    if (smem < need) smem = need;
    if (smem > (size_t)di.max_smem_optin) return cudaErrorNotSupported;
    const void *fn = split  ? (const void *)fwd_tc_bf16_kernel<true>
                     : bf16 ? (const void *)fwd_tc_bf16_kernel<false>
                            : (const void *)fwd_tc_kernel<KIND_TF32>;
    if (!ensure_smem_attr(fn, smem)) return cudaErrorInvalidValue;
    // runs of 8 consecutive entries per CTA (the fan-in of a typical output group) and as
    // many CTAs as that gives: the hardware keeps as many resident as the shared-memory
    // reservation above allows, and that reservation keeps their TMEM within 512 columns
    long long ept = (tune && tune->entries_per_team > 0) ? tune->entries_per_team : 8;
    if (ept < 1) ept = 1;
    if (ept > INT_MAX) ept = INT_MAX;
    a.entries_per_cta = (int)ept;
    const long long grid = (nb + ept - 1) / ept;
    if (grid > INT_MAX) return cudaErrorInvalidValue;
    if (split)
        fwd_tc_bf16_kernel<true><<<(unsigned)grid, kTcThreads, smem, st>>>(a);
    else if (bf16)
        fwd_tc_bf16_kernel<false><<<(unsigned)grid, kTcThreads, smem, st>>>(a);
    else
        fwd_tc_kernel<KIND_TF32><<<(unsigned)grid, kTcThreads, smem, st>>>(a);
    return (int)cudaGetLastError();
}

// Self-test of the bounded wait: an mbarrier that nothing ever arrives on is waited
// for with the kernels' own bounded wait (a short limit); the wait runs out, the
// kernel records code 1 in the device error word and returns, and the context stays
// usable.  No tensor memory, no copies in flight.
__global__ void wait_selftest_kernel()
{
    __shared__ uint64_t mbar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = mbar_wait(smem_u32(&mbar), 0, 1u << 12);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicCAS(&g_tc_error, 0u, 1u);
}

}  // namespace kgb

extern "C" int kronmult_diag_wait_selftest(int *code)
{
    if (!code) return cudaErrorInvalidValue;
    *code = 0;
    const unsigned z = 0;
    cudaError_t e = cudaMemcpyToSymbol(kgb::g_tc_error, &z, sizeof z);
    if (e != cudaSuccess) return e;
    kgb::wait_selftest_kernel<<<1, 32>>>();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
    unsigned v = 0;
    if ((e = cudaMemcpyFromSymbol(&v, kgb::g_tc_error, sizeof v)) != cudaSuccess) return e;
    *code = (int)v;
    return cudaMemcpyToSymbol(kgb::g_tc_error, &z, sizeof z);
}

extern "C" int kronmult_device_error(int *code, int clear)
{
    if (!code) return cudaErrorInvalidValue;
    unsigned v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, kgb::g_tc_error, sizeof v);
    if (e != cudaSuccess) return e;
    *code = (int)v;
    if (clear && v) {
        const unsigned z = 0;
        e = cudaMemcpyToSymbol(kgb::g_tc_error, &z, sizeof z);
    }
    return e;
}
