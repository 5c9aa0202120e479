// Grouped forward: descriptors shared by the planner (grouped.cu) and the per-group
// persistent kernels (grouped_kernels.cuh, instantiated in grouped_inst_*.cu).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "fwd_kernels.cuh"
#include "kronmult_gb300.h"

namespace kgb {

constexpr int kGroupedBlock = 256;  // threads per CTA of the persistent kernels

// One group's persistent launch: teams pull work units (index u, entries
// [u*unit, (u+1)*unit)) from `queue` until n_units are taken.
//
// Deterministic mode (a segmented reduction): the pointer tables are the group's
// tables gathered in sorted order (entries ordered by output pointer on the device,
// ties in entry order) and `keys` holds the sorted output pointers.  A unit sums each
// of its runs of equal output pointers in entry order.  A run that is a whole
// segment (all of that output's entries) is added into the output with one plain
// read-modify-write; a run that continues from the previous unit goes to partial slot
// 2u, one that continues into the next unit (and does not come from the previous
// one) to slot 2u+1 -- N values each.  gq_seg_reduce then adds every segment that
// crosses unit boundaries: its partials in order, into the output once.  The sums are
// independent of scheduling: bitwise reproducible for a given unit size.
struct GqArgs {
    const void *const *mats;
    const void *const *in;
    void *const *out;
    const unsigned long long *keys;      // deterministic mode: sorted output pointers
    void *partial;                       // deterministic mode: 2 * n_units slots of N compute-type values
    unsigned *queue;                     // this group's unit counter (zeroed per run)
    long long nb, unit, n_units;
    int snap;  // deterministic mode, n = 9..16: units moved to segment starts instead of partial slots
    int d, n, stride, N;
    int team_size, team_elems, vec_pad;  // vec_pad: offset of the factors in a team's slice
};

using GqFn = void (*)(const GqArgs);

// Kernel for a group: fibre mapping (compile-time n <= 8, QMAX fibres per thread),
// element mapping with compile-time n (FP64, EMAX outputs per thread), or element
// mapping with n at run time (n = 9..16).  Null when no instantiation fits.
template <typename T, typename TO> GqFn gq_fibre_lookup(int nn, int qmax, bool det);
template <typename T, typename TO> GqFn gq_elem_lookup(int nn, int emax, bool det);
// the element mapping with each thread's factor row in registers (team size a multiple
// of n and of 32; EMAX 2 or 4; n = 4, 8)
template <typename T, typename TO> GqFn gq_elem_rows_lookup(int nn, int emax, bool det);
template <typename T, typename TO> GqFn gq_elem_rt_lookup(int emax, bool det);

// Double-float kernel for a group (FP64 data, FP32-pipe arithmetic; n = 2..8, QMAX
// fibres per thread up to 4).  Null when no instantiation fits.
GqFn gq_df_lookup(int nn, int qmax, bool det);

// deterministic mode, after the group's kernel: the segments that cross unit boundaries
void gq_seg_reduce_launch(const GqArgs &a, int dtype, cudaStream_t st);

// Device-side grouping of one group's entries by output pointer (deterministic mode):
// sorts (pointer, entry index) pairs into keys/perm (m >= nb, a power of two >= 2048),
// then gathers the group's pointer tables in that order into s_mats / s_in / s_out.
void gq_group_launch(const void *const *mats, const void *const *in, const void *const *out, int d, long long nb,
                     long long m, unsigned long long *keys, long long *perm, const void **s_mats,
                     const void **s_in, void **s_out, cudaStream_t st);

struct GqLaunch {
    GqFn fn = nullptr;
    int grid = 0, block = kGroupedBlock;
    size_t smem = 0;
    GqArgs args{};
    // deterministic mode: sort buffers (m = power of two >= nb entries) and the group's
    // pointer tables in sorted order, which the kernel reads
    long long sort_m = 0;
    unsigned long long *keys = nullptr;
    long long *perm = nullptr;
    const void **s_mats = nullptr, **s_in = nullptr;
    void **s_out = nullptr;
    const void *const *mats = nullptr, *const *in = nullptr, *const *out = nullptr;  // the caller's tables
};

struct GqAdjoint {  // one adjoint group, run with the regular adjoint entry point
    kronmult_adjoint_group g{};
};

struct GroupedPlan {
    int dtype = 0, mode = 0, device = 0;
    std::vector<GqLaunch> launches;  // forward groups with entries
    std::vector<GqAdjoint> adjoints;
    unsigned *counters = nullptr;    // one per launch
    void *dmem = nullptr;            // counters and sort buffers, one allocation
    std::vector<cudaStream_t> branches;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    long long n_units = 0, n_sorted = 0;
    int grid_max = 0;
    size_t smem_max = 0;
};

}  // namespace kgb
