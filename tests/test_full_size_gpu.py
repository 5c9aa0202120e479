"""Element-wise parity at the full sizes of the benchmark configurations.

Every output element of the whole batch is compared, not a sample:
  C2  d=6 n=4 stride 8, 36864 entries: the oracle (kronmult_omp restated) and the
      reference's own GPU kernel (kronmult_gpu/kronmult.cu:139-197 built for sm_103a)
  C3  four (d, n) groups, ~420k entries: separate launches and the grouped persistent
      launch in both output modes, against the oracle and the reference kernel
  C4  d=4 n=8, 32768 entries in FP32 storage with FP32 / TF32 / BF16 / split-BF16 contraction and
      FP64 outputs: relative L2 and max error against the FP64 oracle
  C5  d=3 n=6, 16384 entries with shared factors: forward, grad_input (the oracle on
      transposed factors) and grad_A (the mode-unfolding formula) in FP64 and FP32
Tolerances: FP64 relative L2 <= 1e-13 (atomic summation order is the only permitted
difference), FP32 <= 1e-5, TF32 <= 2e-3, BF16 <= 2e-2, split BF16 <= 1e-4 against FP64."""
import functools

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import ref_gpu

pytestmark = pytest.mark.gpu

TOL64 = 1e-13
TOL_COMPUTE = {"fp32": 1e-5, "tf32": 2e-3, "bf16": 2e-2, "bf16x3": 1e-4}


@functools.lru_cache(maxsize=None)
def config(name):
    from kronmult_gb300 import workloads as W

    return getattr(W, name)()


@functools.lru_cache(maxsize=None)
def oracle_out(name, gi=None, dtype="f64"):
    b = config(name) if gi is None else config(name)[gi]
    if dtype == "f64":
        return O.forward(b)
    return O.forward(b, dtype=np.float32, out_dtype=np.float64)


def reference_kernel(db, dtype="f64"):
    """The reference kernel on the batch, adding into zeroed outputs (db.outputs is zeroed)."""
    if not ref_gpu.available():
        pytest.skip("reference cubin not built (the reference sources are needed to build it)")
    from test_reference_gpu import reference_run

    db.outputs.zero_()
    return reference_run(db, dtype).cpu().numpy()


def test_c2_full_f64(cuda):
    from kronmult_gb300 import DeviceBatch

    b = config("config2")
    db = DeviceBatch.from_host(b, device=cuda)
    db.forward(sync=True)
    got = db.outputs.cpu().numpy()
    assert O.rel_l2(got, oracle_out("config2")) <= TOL64
    ref = reference_kernel(db)
    assert O.rel_l2(got, ref) <= TOL64
    assert O.rel_l2(ref, oracle_out("config2")) <= TOL64


@pytest.mark.parametrize("gi", range(4))
def test_c3_full_groups_separate(cuda, gi):
    from kronmult_gb300 import DeviceBatch

    b = config("config3")[gi]
    db = DeviceBatch.from_host(b, device=cuda)
    db.forward(sync=True)
    got = db.outputs.cpu().numpy()
    assert O.rel_l2(got, oracle_out("config3", gi)) <= TOL64
    assert O.rel_l2(reference_kernel(db), got) <= TOL64


@pytest.mark.parametrize("mode", ["atomic", "deterministic"])
def test_c3_full_grouped_graph(cuda, mode):
    """The whole configuration in one persistent launch, replayed from a CUDA graph."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300.grouped import GroupedPlan

    groups = config("config3")
    dbs = [DeviceBatch.from_host(b, device=cuda) for b in groups]
    plan = GroupedPlan(dbs, mode=mode)
    st = torch.cuda.Stream(cuda)
    with torch.cuda.stream(st):
        plan.run(stream=st)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=st):
        plan.run(stream=st)
    first = [db.outputs.cpu().numpy() for db in dbs]
    for db in dbs:
        db.outputs.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for gi, db in enumerate(dbs):
        got = db.outputs.cpu().numpy()
        assert O.rel_l2(got, oracle_out("config3", gi)) <= TOL64
        assert O.rel_l2(first[gi], oracle_out("config3", gi)) <= TOL64
        if mode == "deterministic":
            assert np.array_equal(got, first[gi])
    plan.close()


@pytest.mark.parametrize("compute", ["fp32", "tf32", "bf16", "bf16x3"])
def test_c4_full_reduced_precision(cuda, compute, record_property):
    from kronmult_gb300 import DeviceBatch, _lib, forward_f32_f64out

    code = {"fp32": _lib.KRONMULT_COMPUTE_FP32, "tf32": _lib.KRONMULT_COMPUTE_TF32,
            "bf16": _lib.KRONMULT_COMPUTE_BF16, "bf16x3": _lib.KRONMULT_COMPUTE_BF16X3}[compute]
    b = config("config4")
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64)
    forward_f32_f64out(db, compute=code, sync=True)  # raises if a tensor-core wait ran out
    got = db.outputs.cpu().numpy()
    ref64 = oracle_out("config4")
    err, mx = O.rel_l2(got, ref64), O.max_rel(got, ref64)
    record_property("rel_l2_vs_fp64", err)
    record_property("max_err_vs_fp64", mx)
    print(f"C4 {compute}: relative L2 {err:.3e}, max error {mx:.3e} against FP64")
    assert err <= TOL_COMPUTE[compute]
    if compute == "fp32":
        # the same FP32 sweep per entry as the oracle's, summed in FP64
        assert O.rel_l2(got, oracle_out("config4", dtype="f32")) <= 1e-6


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_c5_full_forward_and_adjoint(cuda, dtype):
    from kronmult_gb300 import DeviceBatch, adjoint

    b = config("config5")
    tol = TOL64 if dtype == torch.float64 else 1e-5
    g = np.random.Generator(np.random.PCG64(1105)).standard_normal((b.n_out, b.N))
    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype)
    db.forward()
    gin = torch.zeros_like(db.inputs)
    gfa = torch.zeros_like(db.factors)
    adjoint(db, torch.from_numpy(g).to(cuda, dtype), gin, gfa)
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.double().cpu().numpy(), oracle_out("config5")) <= tol
    assert O.rel_l2(gin.double().cpu().numpy(), O.forward(O.transposed_batch(b, g))) <= tol
    n, st = b.n, b.stride
    gA = gfa.double().cpu().numpy()[:, :n * st].reshape(-1, n, st)[:, :, :n].transpose(0, 2, 1)
    assert O.rel_l2(gA, O.grad_factors(b, g)) <= tol
    if dtype == torch.float64:
        assert O.rel_l2(reference_kernel(db), oracle_out("config5")) <= TOL64
