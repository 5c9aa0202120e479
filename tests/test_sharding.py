"""Output-group sharding across ranks, with world_size-2 gloo process groups on
CPU: every entry lands on exactly one rank, no output is split, and the gathered
per-rank results (computed with the oracle, standing in for each rank's GPU)
equal the single-process result."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from kronmult_gb300 import workloads as W
from kronmult_gb300.sharding import shard_batch, shard_bounds


def test_bounds_respect_groups():
    b = W.config3(scale=0.01)[1]  # ragged fan-in 1..27
    for world in (1, 2, 3, 8):
        bounds = shard_bounds(b.out_index, world)
        assert bounds[0][0] == 0 and bounds[-1][1] == b.nb
        for (b0, e0), (b1, e1) in zip(bounds, bounds[1:]):
            assert e0 == b1
        owners = {}
        for r in range(world):
            s, outs = shard_batch(b, r, world)
            for o in outs:
                assert o not in owners, "an output vector is split across ranks"
                owners[o] = r
        assert len(owners) == len(np.unique(b.out_index))


def test_bounds_balance():
    b = W.config2(scale=64 / 4096)
    sizes = [e - s for s, e in shard_bounds(b.out_index, 4)]
    assert max(sizes) - min(sizes) <= 9  # one fan-in group


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = W.make_batch(3, 4, 4, 10, np.arange(1, 11), seed=5, out_init="normal")
    shard, outs = shard_batch(b, rank, world)
    y = O.forward(shard)
    full = torch.zeros((b.n_out, b.N), dtype=torch.float64)
    full[torch.from_numpy(outs)] = torch.from_numpy(y)
    mask = torch.zeros(b.n_out, dtype=torch.float64)
    mask[torch.from_numpy(outs)] = 1
    dist.all_reduce(full)
    dist.all_reduce(mask)
    if rank == 0:
        q.put((float(O.rel_l2(full.numpy(), O.forward(b))), mask.numpy().tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    err, mask = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert err <= 1e-15
    assert all(m == 1.0 for m in mask)  # every output owned by exactly one rank


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_shards_through_cuda_union_equals_oracle(cuda, world):
    """The shards bench.py gives each rank (sharding.shard_batch of one seeded batch),
    run one after another through the CUDA forward on one GPU: every output is
    computed by exactly one shard, and the union equals the oracle on the whole batch."""
    import torch

    from kronmult_gb300 import DeviceBatch
    from oracle import oracle as O

    b = W.config3(scale=0.05)[2]  # d=4, n=4, ragged fan-in 1..27
    full = np.full((b.n_out, b.N), np.nan)
    for r in range(world):
        shard, outs = shard_batch(b, r, world)
        db = DeviceBatch.from_host(shard, device=cuda)
        db.forward(sync=True)
        assert np.all(np.isnan(full[outs])), "an output computed by two shards"
        full[outs] = db.outputs.cpu().numpy()
    assert not np.isnan(full).any()
    assert O.rel_l2(full, O.forward(b)) <= 1e-13
