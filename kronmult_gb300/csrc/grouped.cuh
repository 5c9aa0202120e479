// Device-side descriptors of the grouped persistent forward.
#pragma once
#include "fwd_kernels.cuh"
#include "kronmult_gb300.h"

namespace kgb {

constexpr int kGroupedBlock = 256;  // threads per CTA of the persistent kernel

struct GroupDesc {
    const void *const *mats;
    const void *const *in;
    void *const *out;
    const long long *perm;  // entry order (null = identity)
    int d, n, stride, N;
    int team_size, teams_per_cta, team_elems, vec_pad, qmax;
    int emax;  // > 0: element-mapped team forward with this many outputs per thread
};

struct CtaItem {             // one queue item: `count` team ranges of one group
    int group;
    int count;
    long long first_range;
};

struct TeamRange {           // entries [begin, end) in the group's (permuted) order
    long long begin, end;
};

struct GroupedPlan {
    int dtype = 0, mode = 0, device = 0, n_groups = 0;
    int grid = 0, n_items = 0;
    size_t smem = 0;
    long long n_ranges = 0, n_perm = 0;
    const void *fn = nullptr;
    void *dmem = nullptr;  // one allocation holding everything below
    size_t dmem_bytes = 0;
    unsigned *counters = nullptr;
    GroupDesc *groups = nullptr;
    CtaItem *items = nullptr;
    TeamRange *ranges = nullptr;
};

}  // namespace kgb
