"""Partition of a batch across ranks (one GPU per rank).

Entries that add into the same output vector must stay on one rank; then every
rank owns its outputs outright and the forward needs no collective.  A shard is
a contiguous range of entries cut only at output-group boundaries, chosen so that
the shards carry nearly equal numbers of entries (equal work: every entry of a
batch costs the same 2*d*n*N flops).
"""
from __future__ import annotations

import numpy as np

from .workloads import Batch


def group_order(out_index: np.ndarray) -> np.ndarray:
    """Stable order of entries by output vector (identity when groups are contiguous)."""
    return np.argsort(out_index, kind="stable")


def shard_bounds(out_index: np.ndarray, world: int) -> list[tuple[int, int]]:
    """[begin, end) entry ranges (in group order) for `world` ranks, cut at group boundaries."""
    o = np.asarray(out_index)[group_order(out_index)]
    nb = int(o.shape[0])
    starts = np.flatnonzero(np.r_[True, o[1:] != o[:-1]]) if nb else np.zeros(0, dtype=np.int64)
    bounds = []
    b = 0
    for r in range(world):
        if r == world - 1:
            e = nb
        else:
            target = (nb * (r + 1) + world - 1) // world
            # the group start closest to the ideal cut, not before b
            cand = starts[starts >= b]
            e = int(cand[np.argmin(np.abs(cand - target))]) if cand.size else nb
            e = max(e, b)
        bounds.append((b, e))
        b = e
    return bounds


def shard_batch(b: Batch, rank: int, world: int) -> tuple[Batch, np.ndarray]:
    """Return (shard, output ids): the entries of `rank` with their outputs renumbered
    0..E_r-1, and the original ids of those outputs."""
    order = group_order(b.out_index)
    lo, hi = shard_bounds(b.out_index, world)[rank]
    sel = order[lo:hi]
    outs, local = np.unique(b.out_index[sel], return_inverse=True)
    fsets, flocal = np.unique(b.fac_index[sel], return_inverse=True)
    fac_rows = (fsets[:, None] * b.d + np.arange(b.d)[None, :]).reshape(-1)
    shard = Batch(f"{b.name}_r{rank}of{world}", b.d, b.n, b.stride, b.block, b.factors[fac_rows],
                  b.inputs[sel], b.out_init[outs], flocal.astype(np.int64), local.astype(np.int64), dict(b.meta))
    return shard, outs
