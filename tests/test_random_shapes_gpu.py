"""Seeded random sweep over shapes, strides, ragged fan-ins, output aliasing orders,
precisions and entry points, each against the oracle.  Every planner path (single
entry, element mapping, runs, two modes per pass, two-pass and global sweeps, the
generic kernel, tensor cores, emulated FP64, indexed) is reached by some case."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-13, torch.float32: 1e-5}


def random_case(seed):
    from kronmult_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(rng.integers(1, 11))
    max_d = max(1, int(np.floor(np.log(40000) / np.log(max(n, 2)))))
    d = int(rng.integers(0 if n > 1 else 1, min(max_d, 7) + 1))
    stride = n + int(rng.integers(0, 3))
    n_out = int(rng.integers(1, 9))
    fan = rng.integers(1, 6, size=n_out)
    b = W.make_batch(d, n, stride, n_out, fan, seed=seed, shared_factors=bool(rng.integers(0, 2)),
                     out_init="normal")
    if rng.integers(0, 2):  # outputs visited in a shuffled order (non-contiguous aliasing)
        perm = rng.permutation(b.nb)
        b = W.Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs[perm], b.out_init,
                    b.fac_index[perm], b.out_index[perm])
    return b


@pytest.mark.parametrize("seed", list(range(24)))
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_random_forward(cuda, seed, dtype):
    from kronmult_gb300 import DeviceBatch

    b = random_case(4000 + seed)
    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype, with_workspace=True)
    db.forward(sync=True)
    assert O.rel_l2(db.outputs.double().cpu().numpy(), O.forward(b)) <= TOL[dtype]


@pytest.mark.parametrize("seed", list(range(12)))
def test_random_emulated_and_indexed(cuda, seed):
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300.api import forward_f64_emulated, forward_indexed

    b = random_case(5000 + seed)
    ref = O.forward(b)
    if 2 <= b.n <= 8 and b.d >= 1:
        db = DeviceBatch.from_host(b, device=cuda, with_workspace=True)
        forward_f64_emulated(db)
        torch.cuda.synchronize()
        assert O.rel_l2(db.outputs.cpu().numpy(), ref) <= 1e-13
    fac = torch.from_numpy(b.factors).to(cuda)
    x = torch.from_numpy(b.inputs).to(cuda)
    y = torch.from_numpy(b.out_init).to(cuda)
    fidx = torch.from_numpy(b.fac_index[:, None] * b.d + np.arange(b.d)[None, :]).to(cuda)
    if b.d == 0:
        fidx = torch.zeros((b.nb, 0), dtype=torch.int64, device=cuda)
    forward_indexed(b.d, b.n, b.stride, fac, fidx, x, y, torch.from_numpy(b.out_index).to(cuda))
    torch.cuda.synchronize()
    assert O.rel_l2(y.cpu().numpy(), ref) <= 1e-13


@pytest.mark.parametrize("seed", list(range(8)))
def test_random_fp32_f64out(cuda, seed):
    """FP32 storage with FP32 contraction into FP64 outputs; TF32 / BF16 where n = 8."""
    from kronmult_gb300 import DeviceBatch, _lib
    from kronmult_gb300.api import forward_f32_f64out

    b = random_case(6000 + seed)
    ref = O.forward(b)
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64, with_workspace=True)
    forward_f32_f64out(db, compute=_lib.KRONMULT_COMPUTE_FP32)
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.cpu().numpy(), ref) <= 1e-5
