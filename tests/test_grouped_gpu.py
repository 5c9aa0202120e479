"""Grouped persistent forward (atomic and deterministic modes), CUDA-graph
capture, and the autotuner, against the C oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL64 = 1e-13


def device_groups(batches, cuda, dtype=torch.float64):
    from kronmult_gb300 import DeviceBatch

    return [DeviceBatch.from_host(b, device=cuda, dtype=dtype) for b in batches]


def scrambled(b, seed):
    """Same batch with outputs assigned non-contiguously (random entry order)."""
    from kronmult_gb300.workloads import Batch

    p = np.random.Generator(np.random.PCG64(seed)).permutation(b.nb)
    return Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs[p], b.out_init, b.fac_index[p],
                 b.out_index[p])


@pytest.mark.parametrize("mode", ["atomic", "deterministic"])
def test_config3_groups(cuda, mode):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = W.config3(scale=0.05)
    dbs = device_groups(batches, cuda)
    plan = GroupedPlan(dbs, mode=mode)
    plan.run()
    torch.cuda.synchronize()
    for b, db in zip(batches, dbs):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
    info = plan.info()
    assert info["items"] > 0 and info["grid"] > 0 and info["block"] == 256


def test_deterministic_is_bitwise_reproducible(cuda):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = [scrambled(b, 3 + i) for i, b in enumerate(W.config3(scale=0.02))]
    results = []
    for rep in range(3):
        dbs = device_groups(batches, cuda)
        plan = GroupedPlan(dbs, mode="deterministic")
        assert plan.info()["permuted"] == sum(b.nb for b in batches)  # outputs were not contiguous
        plan.run()
        torch.cuda.synchronize()
        results.append([db.outputs.cpu().numpy().copy() for db in dbs])
    for b, r in zip(batches, results[0]):
        assert O.rel_l2(r, O.forward(b)) <= TOL64
    for other in results[1:]:
        for a, c in zip(results[0], other):
            assert np.array_equal(a, c)


def test_deterministic_matches_entry_order_sum(cuda):
    """Each output is out_init + (((y_0 + y_1) + y_2) + ...) over its entries in order."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan
    from kronmult_gb300.workloads import Batch

    b = W.make_batch(3, 4, 4, 5, 6, seed=12, out_init="normal")
    db = device_groups([b], cuda)[0]
    GroupedPlan([db], mode="deterministic").run()
    torch.cuda.synchronize()
    per_entry = O.forward(Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, np.zeros((b.nb, b.N)),
                                b.fac_index, np.arange(b.nb, dtype=np.int64)))
    want = b.out_init.copy()
    for e in range(b.n_out):
        ks = np.nonzero(b.out_index == e)[0]
        acc = per_entry[ks[0]].copy()
        for k in ks[1:]:
            acc = acc + per_entry[k]
        want[e] = want[e] + acc
    # per-entry sweeps agree to rounding (FMA contraction); the association is the same
    assert O.rel_l2(db.outputs.cpu().numpy(), want) <= 1e-15


def test_graph_capture_replay(cuda):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = W.config3(scale=0.02)
    dbs = device_groups(batches, cuda)
    plan = GroupedPlan(dbs, mode="deterministic")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan.run(stream=s)  # warm-up outside the capture
    torch.cuda.synchronize()
    for db in dbs:
        db.outputs.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.run(stream=s)
    torch.cuda.synchronize()
    for db in dbs:
        db.outputs.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for b, db in zip(batches, dbs):
        want = 2 * O.forward(b)
        assert O.rel_l2(db.outputs.cpu().numpy(), want) <= TOL64


def test_grouped_f32(cuda):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = W.config3(scale=0.02)
    dbs = device_groups(batches, cuda, dtype=torch.float32)
    GroupedPlan(dbs, mode="atomic").run()
    torch.cuda.synchronize()
    for b, db in zip(batches, dbs):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= 1e-5


def test_shared_output_across_groups_rejected(cuda):
    import kronmult_gb300 as K
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = W.make_batch(2, 4, 4, 2, 3, seed=1)
    db1, db2 = device_groups([b, b], cuda)
    db2.out_ptrs = db1.out_ptrs.clone()
    with pytest.raises(K.KronmultError):
        GroupedPlan([db1, db2], mode="deterministic")
    GroupedPlan([db1, db2], mode="atomic")  # allowed with atomics


def test_autotune_and_cache(cuda, tmp_path):
    from kronmult_gb300 import DeviceBatch, _lib
    from kronmult_gb300 import grouped as G
    from kronmult_gb300 import workloads as W

    G.tuning_cache_clear()
    best, ms = G.autotune_forward(3, 4, _lib.KRONMULT_DTYPE_F64, nb_sample=4096)
    assert best["team_size"] in (8, 16, 32, 64, 128, 256, 512) and ms > 0
    assert G.tuning_cache_get(3, 4, _lib.KRONMULT_DTYPE_F64) == best
    path = str(tmp_path / "tune.txt")
    G.tuning_cache_save(path)
    G.tuning_cache_clear()
    assert G.tuning_cache_get(3, 4, _lib.KRONMULT_DTYPE_F64) is None
    G.tuning_cache_load(path)
    assert G.tuning_cache_get(3, 4, _lib.KRONMULT_DTYPE_F64) == best
    b = W.config1(scale=16 / 1024)
    db = DeviceBatch.from_host(b, device=cuda)
    db.forward(sync=True)  # uses the cached shape
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
    G.tuning_cache_clear()


def test_autotune_grouped_tunings_give_correct_results(cuda):
    """Per-group team sizes picked by timing the persistent kernel; the plan built
    with them matches the oracle and the outputs are left as they were by the search."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import grouped as G
    from kronmult_gb300 import workloads as W

    groups = W.config3(scale=40 / 8000)
    dbs = [DeviceBatch.from_host(b, device=cuda) for b in groups]
    tunings = G.autotune_grouped(dbs, mode="atomic", reps=2)
    assert len(tunings) == len(groups)
    for db, b in zip(dbs, groups):
        assert torch.equal(db.outputs.cpu(), torch.from_numpy(b.out_init))
    plan = G.GroupedPlan(dbs, mode="atomic", tunings=tunings)
    plan.run()
    torch.cuda.synchronize()
    for db, b in zip(dbs, groups):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= 1e-13
    plan.close()
