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
    assert info["items"] > 0 and info["grid"] > 0 and 32 <= info["block"] <= 256 and info["block"] % 32 == 0


def test_deterministic_is_bitwise_reproducible(cuda):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = [scrambled(b, 3 + i) for i, b in enumerate(W.config3(scale=0.02))]
    results = []
    for rep in range(3):
        dbs = device_groups(batches, cuda)
        plan = GroupedPlan(dbs, mode="deterministic")
        assert plan.info()["sorted"] == sum(b.nb for b in batches)  # ordered on the device
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


def test_shared_output_across_groups(cuda):
    """Two groups adding into the same outputs: the deterministic mode runs the groups
    one after another, so the sum is right and bitwise the same on every run; the
    atomic mode is right up to summation order."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = W.make_batch(2, 4, 4, 2, 3, seed=1)
    db1, db2 = device_groups([b, b], cuda)
    db2.out_ptrs = db1.out_ptrs.clone()  # both groups add into db1's outputs
    want = 2 * O.forward(b)
    runs = []
    for mode in ("deterministic", "deterministic", "atomic"):
        db1.outputs.zero_()
        GroupedPlan([db1, db2], mode=mode).run()
        torch.cuda.synchronize()
        runs.append(db1.outputs.cpu().numpy())
        assert O.rel_l2(runs[-1], want) <= TOL64
    assert np.array_equal(runs[0], runs[1])


def reference_aliasing(b, distinct):
    """The reference tests' output map (tests/utils/utils_cpu.h:79-83): entry i < distinct
    adds into output i, every other entry into output (i*distinct)//nb -- not contiguous."""
    from kronmult_gb300.workloads import Batch

    idx = np.arange(b.nb, dtype=np.int64)
    out_index = np.where(idx < distinct, idx, (idx * distinct) // b.nb)
    return Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, b.out_init[:distinct], b.fac_index,
                 out_index)


@pytest.mark.parametrize("d,n,nb", [(3, 4, 3903), (2, 8, 1000), (4, 6, 700), (2, 12, 300)])
def test_deterministic_reference_aliasing_bitwise(cuda, d, n, nb):
    """The reference's non-contiguous aliasing (5 outputs, long runs, entries 0..4 apart
    from the rest): ordered by output pointer on the device and summed by the segmented
    reduction -- the oracle's result, bitwise the same on every plan with the same unit
    size and every run; other unit sizes group the sums differently (agreement to
    rounding)."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = reference_aliasing(W.make_batch(d, n, n + 3, nb, 1, seed=3900 + d, out_init="normal"), 5)
    want = O.forward(b)
    results = []
    for unit in (37, 37, 37, 5, 0):
        db = device_groups([b], cuda)[0]
        plan = GroupedPlan([db], mode="deterministic", tunings=[{"entries_per_team": unit}])
        plan.run()
        plan.run()  # a second run adds the same values again
        torch.cuda.synchronize()
        results.append(db.outputs.cpu().numpy())
        assert O.rel_l2(results[-1], 2 * want - b.out_init) <= TOL64
        plan.close()
    assert np.array_equal(results[0], results[1]) and np.array_equal(results[0], results[2])


@pytest.mark.parametrize("captured", [False, True])
def test_regroup_after_table_change(cuda, captured):
    """An output pointer table changed in place: kronmult_grouped_regroup (on a stream,
    optionally captured in the same graph as the run) re-orders the entries on the
    device and the next run uses the new assignment."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan
    from kronmult_gb300.workloads import Batch

    b = W.make_batch(3, 5, 6, 40, 6, seed=77)
    db = device_groups([b], cuda)[0]
    plan = GroupedPlan([db], mode="deterministic")
    perm = np.random.Generator(np.random.PCG64(78)).permutation(b.nb)
    b2 = Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, b.out_init, b.fac_index, b.out_index[perm])
    new_ptrs = db.outputs.data_ptr() + torch.from_numpy(b2.out_index).to(cuda) * (db.outputs.shape[1] * 8)
    s = torch.cuda.Stream()
    db.out_ptrs.copy_(new_ptrs)  # same tensor, new contents
    torch.cuda.synchronize()
    db.outputs.zero_()
    if captured:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            plan.regroup(stream=s)
            plan.run(stream=s)
        db.outputs.zero_()
        g.replay()
    else:
        with torch.cuda.stream(s):
            plan.regroup(stream=s)
            plan.run(stream=s)
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b2)) <= TOL64


@pytest.mark.parametrize("mode", ["atomic", "deterministic"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_runtime_n_groups(cuda, mode, dtype):
    """n = 9..16 groups (n taken at run time) beside compile-time ones."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = [W.make_batch(2, 12, 13, 6, 4, seed=81), W.make_batch(3, 4, 4, 9, 3, seed=82),
               W.make_batch(2, 9, 9, 5, 5, seed=83)]
    dbs = device_groups(batches, cuda, dtype=dtype)
    GroupedPlan(dbs, mode=mode).run()
    torch.cuda.synchronize()
    tol = TOL64 if dtype == torch.float64 else 1e-5
    for b, db in zip(batches, dbs):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= tol


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-13), (torch.float32, 1e-5)])
def test_forward_and_adjoint_groups_in_one_graph(cuda, dtype, tol):
    """A plan with a forward group and an adjoint group (the configuration-5 shape with
    shared factors), captured in one graph: outputs against the oracle, grad_input
    against the oracle on transposed factors, grad_A against the mode-unfolding formula."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = W.config5(scale=64 / 2048)
    g = np.random.Generator(np.random.PCG64(1106)).standard_normal((b.n_out, b.N))
    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype)
    gt = torch.from_numpy(g).to(cuda, dtype)
    gin = torch.zeros_like(db.inputs)
    gfa = torch.zeros_like(db.factors)
    plan = GroupedPlan([db], mode="atomic", adjoints=[(db, gt, gin, gfa)])
    assert plan.info()["kernels"] == 2
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        plan.run(stream=s)  # warm-up outside the capture
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=s):
        plan.run(stream=s)
    for t in (db.outputs, gin, gfa):
        t.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.double().cpu().numpy(), O.forward(b)) <= tol
    assert O.rel_l2(gin.double().cpu().numpy(), O.forward(O.transposed_batch(b, g))) <= tol
    n, st = b.n, b.stride
    gA = gfa.double().cpu().numpy()[:, :n * st].reshape(-1, n, st)[:, :, :n].transpose(0, 2, 1)
    assert O.rel_l2(gA, O.grad_factors(b, g)) <= tol
    plan.close()


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


@pytest.mark.parametrize("mode", ["atomic", "deterministic"])
def test_emulated_groups(cuda, mode):
    """arithmetic="emulated": every group's mode products in double-float arithmetic on
    the FP32 pipe; FP64-accurate (relative L2 <= 1e-13 against the oracle), scrambled
    outputs, the deterministic mode bitwise the same on every replay."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = [scrambled(b, 40 + i) for i, b in enumerate(W.config3(scale=0.03))]
    dbs = device_groups(batches, cuda)
    plan = GroupedPlan(dbs, mode=mode, arithmetic="emulated")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan.run(stream=s)
    torch.cuda.synchronize()
    first = [db.outputs.clone() for db in dbs]
    for b, got in zip(batches, first):
        assert O.rel_l2(got.cpu().numpy(), O.forward(b)) <= TOL64
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.run(stream=s)
    for db in dbs:
        db.outputs.zero_()
    g.replay()
    torch.cuda.synchronize()
    for b, db, f in zip(batches, dbs, first):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
        if mode == "deterministic":
            assert torch.equal(db.outputs, f)
    plan.close()


def test_emulated_groups_with_adjoint_and_limits(cuda):
    """An emulated forward group and a native FP64 adjoint group in one plan; n > 8 and
    float32 groups are refused for the emulated arithmetic."""
    from kronmult_gb300 import _lib, adjoint
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = W.make_batch(3, 6, 6, 16, 4, seed=4100)
    db, dba = device_groups([b, b], cuda)
    g = torch.from_numpy(np.random.Generator(np.random.PCG64(4101)).standard_normal((b.n_out, b.N))).to(cuda)
    gin = torch.zeros_like(dba.inputs)
    gfa = torch.zeros_like(dba.factors)
    plan = GroupedPlan([db], mode="atomic", adjoints=[(dba, g, gin, gfa)], arithmetic="emulated")
    plan.run()
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
    gin2 = torch.zeros_like(dba.inputs)
    gfa2 = torch.zeros_like(dba.factors)
    adjoint(dba, g, gin2, gfa2)
    torch.cuda.synchronize()
    assert O.rel_l2(gin.cpu().numpy(), gin2.cpu().numpy()) <= TOL64
    plan.close()
    big = device_groups([W.make_batch(2, 9, 9, 4, 1, seed=4102)], cuda)
    with pytest.raises(_lib.KronmultError):
        GroupedPlan(big, arithmetic="emulated")
    with pytest.raises(TypeError):
        GroupedPlan(device_groups([b], cuda, dtype=torch.float32), arithmetic="emulated")


def test_ctas_per_sm_caps_the_persistent_grid(cuda):
    """kronmult_tuning.ctas_per_sm bounds a group's persistent CTAs per SM; the result is
    unchanged up to summation order."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    batches = W.config3(scale=0.01)
    dbs = device_groups(batches, cuda)
    sms = torch.cuda.get_device_properties(cuda).multi_processor_count
    plan = GroupedPlan(dbs, mode="atomic", tunings=[{"ctas_per_sm": 2}] * len(dbs))
    assert plan.info()["grid"] <= 2 * sms
    plan.run()
    torch.cuda.synchronize()
    for b, db in zip(batches, dbs):
        assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
    plan.close()


def test_emulated_deterministic_regroup(cuda):
    """The double-float plans share the device ordering: after an output table changes in
    place, regroup + run gives the new assignment, bitwise the same on a second run."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan
    from kronmult_gb300.workloads import Batch

    b = W.make_batch(3, 6, 6, 30, 7, seed=91)
    db = device_groups([b], cuda)[0]
    plan = GroupedPlan([db], mode="deterministic", arithmetic="emulated")
    perm = np.random.Generator(np.random.PCG64(92)).permutation(b.nb)
    b2 = Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, b.out_init, b.fac_index, b.out_index[perm])
    db.out_ptrs.copy_(db.outputs.data_ptr() + torch.from_numpy(b2.out_index).to(cuda) * (db.outputs.shape[1] * 8))
    torch.cuda.synchronize()
    outs = []
    for _ in range(2):
        db.outputs.zero_()
        plan.regroup()
        plan.run()
        torch.cuda.synchronize()
        outs.append(db.outputs.clone())
    assert torch.equal(outs[0], outs[1])
    assert O.rel_l2(outs[0].cpu().numpy(), O.forward(b2)) <= TOL64
    plan.close()
