"""FP64-accurate forward in double-float arithmetic (kronmult_batched_f64_emulated_async):
same contract as the native FP64 path, relative L2 <= 1e-13 against the FP64 oracle,
for every supported n, the benchmark shapes, and inputs whose magnitudes span
hundreds of binary orders."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL64 = 1e-13


def run_df(b, cuda, ws=False):
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300.api import forward_f64_emulated

    db = DeviceBatch.from_host(b, device=cuda, with_workspace=ws)
    forward_f64_emulated(db)
    torch.cuda.synchronize()
    return db.outputs.cpu().numpy()


@pytest.mark.parametrize("d,n", [(1, 2), (5, 2), (4, 3), (3, 4), (6, 4), (2, 5), (3, 6), (2, 7), (2, 8), (4, 8)])
def test_df_shapes(cuda, d, n):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 1, 5, 4, seed=700 + 10 * d + n, out_init="normal")
    assert O.rel_l2(run_df(b, cuda), O.forward(b)) <= TOL64


def test_df_config_shapes(cuda):
    from kronmult_gb300 import workloads as W

    for b in (W.config1(scale=32 / 1024), W.config2(scale=16 / 4096), W.config5(scale=16 / 2048)):
        assert O.rel_l2(run_df(b, cuda), O.forward(b)) <= TOL64


def test_df_wide_dynamic_range(cuda):
    """Entries scaled by up to 2^+-250 and factors by up to 2^+-50 (products up to
    2^+-400, far outside FP32's range): the per-entry and per-factor power-of-two
    scaling keeps every double-float value in FP32 range."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(3, 4, 4, 6, 3, seed=77)
    rng = np.random.Generator(np.random.PCG64(78))
    b.inputs = b.inputs * np.exp2(rng.integers(-250, 250, size=(b.nb, 1)).astype(np.float64))
    b.factors = b.factors * np.exp2(rng.integers(-50, 50, size=(b.factors.shape[0], 1)).astype(np.float64))
    got = run_df(b, cuda)
    want = O.forward(b)
    # each output mixes entries of very different magnitudes: compare per output vector
    for e in range(b.n_out):
        assert O.rel_l2(got[e], want[e]) <= TOL64


def test_df_zeros_and_nonfinite(cuda):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(2, 4, 4, 3, 1, seed=79)
    b.inputs[0] = 0.0
    b.inputs[1, 3] = np.inf
    got = run_df(b, cuda)
    want = O.forward(b)
    assert np.array_equal(got[0], want[0])  # zero vector -> zero contribution
    assert not np.isfinite(got[1]).all() and not np.isfinite(want[1]).all()
    assert O.rel_l2(got[2], want[2]) <= TOL64


@pytest.mark.parametrize("d,n,stride", [(5, 8, 8), (10, 3, 4), (8, 4, 5), (7, 5, 5), (16, 2, 2), (7, 6, 6), (5, 7, 7)])
def test_df_two_pass(cuda, d, n, stride):
    """Vectors beyond one team's shared memory: two passes through the workspace,
    chunks and tiles each with their own power-of-two scale."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, stride, 3, 2, seed=760 + 10 * d + n, out_init="normal")
    db = DeviceBatch.from_host(b, device=cuda, with_workspace=True)
    x0 = db.inputs.clone()
    from kronmult_gb300.api import forward_f64_emulated

    forward_f64_emulated(db)
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64
    assert torch.equal(db.inputs, x0)


def test_df_two_pass_published_shape_wide_range(cuda):
    """The published n = 8, d = 6 shape (stride 67, 5 aliased outputs) with inputs
    spanning 2^-300 .. 2^300 across entries and positions."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(6, 8, 67, 5, 2, seed=3904)
    rng = np.random.Generator(np.random.PCG64(3905))
    b.inputs = b.inputs * np.exp2(rng.integers(-300, 300, size=(b.nb, 1)))
    assert O.rel_l2(run_df(b, cuda, ws=True), O.forward(b)) <= TOL64


def test_df_large_without_workspace_is_not_supported(cuda):
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import forward_f64_emulated
    from kronmult_gb300._lib import KronmultError

    b = W.make_batch(5, 8, 8, 1, 1, seed=3906)
    db = DeviceBatch.from_host(b, device=cuda)
    with pytest.raises(KronmultError):
        forward_f64_emulated(db)
