// Process-wide cache of autotuned launch shapes, keyed by (d, n, dtype) on the
// current GPU model.  Filled by kronmult_autotune_forward or loaded from a file;
// consulted by the forward planner and the grouped planner when the caller
// passes no explicit tuning.
#pragma once
#include "kronmult_gb300.h"

namespace kgb {
bool tuning_cache_lookup(int d, int n, int dtype, kronmult_tuning &out);
void tuning_cache_store(int d, int n, int dtype, const kronmult_tuning &t);
}  // namespace kgb
