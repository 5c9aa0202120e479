// Grouped persistent forward in double-float arithmetic (KRONMULT_DTYPE_F64_EMULATED):
// FP64 factors, inputs and outputs, every mode product computed on the FP32 pipe as in
// kronmult_batched_f64_emulated_async (df_common.cuh), one kernel per group compiled for
// its n, pulling work units from the group's device queue like the native grouped
// kernels (grouped_kernels.cuh).  No reference counterpart: the reference serves one
// (d, n) per call in native FP64 (kronmult_gpu/kronmult.cu:173-197).
#include "df_common.cuh"
#include "grouped_kernels.cuh"

namespace kgb {

// One team per entry at a time, whole fibres per thread (df_team), the slice laid out
// as df_entry wants it; deterministic mode keeps its N run sums (FP64) after the slice.
template <int NN, int QMAX, bool DET>
__global__ void __launch_bounds__(kGroupedBlock, 3) gq_df_kernel(const GqArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_unit[kGroupedBlock / 8];
    __shared__ int s_red[kGroupedBlock / 8 * 32];  // per team: reduction space
    const Team tm(a.team_size);
    constexpr int NN2 = NN * NN;
    float *xh = reinterpret_cast<float *>(smem_raw) + (size_t)tm.id * a.team_elems;
    float *xl = xh + a.vec_pad;
    float *mh = xl + a.vec_pad;
    float *ml = mh + a.d * NN2;
    int *fexp = reinterpret_cast<int *>(ml + a.d * NN2);
    double *acc = reinterpret_cast<double *>(xh + df_slice_floats(a.d, NN, a.vec_pad));
    const double *const *mats = reinterpret_cast<const double *const *>(a.mats);
    const double *const *in = reinterpret_cast<const double *const *>(a.in);
    double *const *out = reinterpret_cast<double *const *>(a.out);
    long long b, e;
    unsigned claim = gq_first_claim(a, tm);
    while (gq_next(a, &s_unit[tm.id], tm, claim, b, e)) {
        long long rs = b;
        for (long long ei = b; ei < e; ++ei) {
            bool first, last;
            double *part = gq_run_edges<double, DET>(a, b, e, ei, rs, first, last);
            double *o = out[ei];
            df_entry<NN, QMAX>(in[ei], mats + ei * a.d, a.d, a.stride, a.N, xh, xl, mh, ml, fexp, s_red + tm.id * 32,
                               tm, [&](int p, double v) { gq_add<double, double, DET>(o, acc, part, p, v, first, last); });
        }
    }
}

GqFn gq_df_lookup(int nn, int qmax, bool det)
{
#define KGB_GQDF(NN, Q)                                                \
    case NN * 32 + Q * 2: return gq_df_kernel<NN, Q, false>;           \
    case NN * 32 + Q * 2 + 1: return gq_df_kernel<NN, Q, true>;
#define KGB_GQDF_N(NN) KGB_GQDF(NN, 1) KGB_GQDF(NN, 2) KGB_GQDF(NN, 4)
    switch (nn * 32 + qmax * 2 + (det ? 1 : 0)) {
        KGB_GQDF_N(2) KGB_GQDF_N(3) KGB_GQDF_N(4) KGB_GQDF_N(5) KGB_GQDF_N(6) KGB_GQDF_N(7) KGB_GQDF_N(8)
    default: return nullptr;
    }
#undef KGB_GQDF_N
#undef KGB_GQDF
}

}  // namespace kgb
