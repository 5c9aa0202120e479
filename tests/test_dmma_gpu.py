"""The FP64 forward on the FP64 tensor path (mma m8n8k4, fwd_dmma_kernel and
fwd_dmma_global_kernel) against the FP64 FMA-pipe kernels and the oracle.

Each m8n8k4 MMA computes its elements as the k-ascending FMA chain, so per entry the
tensor path gives bitwise the values of the FMA-pipe kernels (and of the reference
kernel, kronmult_gpu/kronmult.cu:139-197): with one output per entry the outputs are
identical bit for bit; with shared outputs only the order of the atomic additions
differs (relative L2 <= 1e-13 against the oracle)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-13
FMA = {"fp64_path": 1}
TENSOR = {"fp64_path": 2}


def _run(b, cuda, tuning, ws=False):
    from kronmult_gb300 import DeviceBatch

    db = DeviceBatch.from_host(b, device=cuda, with_workspace=ws)
    db.forward(tuning=tuning, sync=True)
    return db.outputs.clone()


@pytest.mark.parametrize("d,n,stride", [(1, 8, 8), (2, 8, 8), (3, 8, 9), (4, 8, 8), (2, 7, 7), (3, 7, 10),
                                        (4, 7, 7), (2, 6, 6), (3, 6, 8), (4, 6, 6), (1, 16, 16), (2, 16, 17),
                                        (3, 16, 16), (1, 7, 7), (1, 6, 6)])
def test_tensor_path_bitwise_per_entry(cuda, d, n, stride):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, stride, 37, 1, seed=7100 + 10 * d + n)  # one output per entry
    got = _run(b, cuda, TENSOR)
    want = _run(b, cuda, FMA)
    assert torch.equal(got, want)
    assert O.rel_l2(got.cpu().numpy(), O.forward(b)) <= TOL64


@pytest.mark.parametrize("d,n,fan", [(2, 8, 9), (3, 8, 8), (4, 8, 27), (3, 7, 5), (3, 16, 4)])
def test_tensor_path_shared_outputs(cuda, d, n, fan):
    from kronmult_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(7200 + d * 10 + n))
    fans = rng.integers(1, fan + 1, size=24)
    b = W.make_batch(d, n, n, 24, fans, seed=7300 + d * 10 + n, out_init="normal")
    got = _run(b, cuda, TENSOR)
    assert O.rel_l2(got.cpu().numpy(), O.forward(b)) <= TOL64


@pytest.mark.parametrize("d,n,stride,nb", [(5, 8, 8, 5), (5, 8, 11, 3), (4, 16, 16, 2)])
def test_tensor_global_sweep_bitwise(cuda, d, n, stride, nb):
    """Vectors beyond shared memory: the tensor-path sweep through input and workspace
    against the FMA-pipe sweep (n = 8) or the generic kernel (n = 16), bit for bit."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, stride, nb, 1, seed=7400 + d * 10 + n)
    got = _run(b, cuda, TENSOR, ws=True)
    want = _run(b, cuda, FMA, ws=True)
    assert torch.equal(got, want)
    if n ** d <= 40000:
        assert O.rel_l2(got.cpu().numpy(), O.forward(b)) <= TOL64


@pytest.mark.parametrize("d,n", [(3, 8), (2, 16)])
def test_automatic_choice_same_bits(cuda, d, n):
    """Whatever unit the automatic choice takes (the FMA pipe for n <= 8, the tensor path
    for n = 16), its bits are those of both explicit choices."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n, 64, 1, seed=7500 + n)
    auto = _run(b, cuda, None)
    assert torch.equal(auto, _run(b, cuda, TENSOR))
    assert torch.equal(auto, _run(b, cuda, FMA))


def test_tensor_path_nonfinite_inputs(cuda):
    """An infinite input value reaches the same outputs through either unit (padding
    products are 0 * 0, so no NaN appears where the FMA chain has none)."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(2, 7, 7, 8, 1, seed=7600)
    b.inputs[0, 3] = np.inf
    b.inputs[5, 10] = -np.inf
    got = _run(b, cuda, TENSOR).cpu().numpy()
    want = _run(b, cuda, FMA).cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(want))
    fin = np.isfinite(want)
    assert np.array_equal(got[fin], want[fin])
    assert np.array_equal(np.isinf(got), np.isinf(want))


def test_mma_rounds_as_the_ascending_fma_chain(cuda):
    """The fact the tensor path rests on: every element of an m8n8k4 .f64 MMA equals the
    k-ascending FMA chain from C (operands of mixed magnitude), and not a different order."""
    import ctypes

    from kronmult_gb300 import _lib

    cnt = (ctypes.c_ulonglong * 3)()
    assert _lib.lib().kronmult_diag_fp64_mma_rounding(cnt) == 0
    assert cnt[2] == 524288
    assert cnt[0] == cnt[2]
    assert cnt[1] < cnt[2] * 0.9


@pytest.mark.parametrize("d,n", [(6, 3), (4, 4), (3, 6), (2, 8)])
def test_fp64_mappings_same_bits(cuda, d, n):
    """kronmult_tuning.fp64_path 3 (whole fibres per thread) and 4 (one output element per
    thread) on the FMA pipe, single call and grouped plan: the same k-ascending chains, so
    with one output per entry every choice gives the same bits."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.grouped import GroupedPlan

    b = W.make_batch(d, n, n, 50, 1, seed=7700 + 10 * d + n)
    outs = [_run(b, cuda, t) for t in (None, {"fp64_path": 3}, {"fp64_path": 4})]
    for t in ({"fp64_path": 3}, {"fp64_path": 4}):
        db = DeviceBatch.from_host(b, device=cuda)
        plan = GroupedPlan([db], mode="atomic", tunings=[t])
        plan.run()
        torch.cuda.synchronize()
        outs.append(db.outputs.clone())
        plan.close()
    for o in outs[1:]:
        assert torch.equal(o, outs[0])
    assert O.rel_l2(outs[0].cpu().numpy(), O.forward(b)) <= TOL64
