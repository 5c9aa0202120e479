"""Indexed forward (integer maps over dense factor/input/output arrays) against
the oracle, including shared factor sets, an input index map and aliasing."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-13), (torch.float32, 1e-5)])
@pytest.mark.parametrize("cfg", ["c1", "c5", "c2"])
def test_indexed_matches_oracle(cuda, dtype, tol, cfg):
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import forward_indexed

    b = {"c1": W.config1(scale=32 / 1024), "c5": W.config5(scale=16 / 2048), "c2": W.config2(scale=8 / 4096)}[cfg]
    fac = torch.from_numpy(b.factors).to(cuda, dtype)
    x = torch.from_numpy(b.inputs).to(cuda, dtype)
    y = torch.from_numpy(b.out_init).to(cuda, dtype)
    fidx = torch.from_numpy(b.fac_index[:, None] * b.d + np.arange(b.d)[None, :]).to(cuda)
    keep = forward_indexed(b.d, b.n, b.stride, fac, fidx, x, y, torch.from_numpy(b.out_index).to(cuda))
    torch.cuda.synchronize()
    assert O.rel_l2(y.cpu().numpy(), O.forward(b)) <= tol
    del keep


def test_indexed_input_map_and_aliasing(cuda):
    """Several entries reading one input row through input_index, outputs aliased
    non-contiguously."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import forward_indexed

    b = W.make_batch(3, 4, 5, 4, 5, seed=81, out_init="normal")
    rng = np.random.Generator(np.random.PCG64(82))
    in_map = rng.integers(0, 3, size=b.nb)
    out_map = rng.integers(0, b.n_out, size=b.nb)
    b2 = W.Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs[in_map], b.out_init, b.fac_index, out_map)
    fac = torch.from_numpy(b.factors).to(cuda)
    x = torch.from_numpy(b.inputs[:3]).to(cuda)
    y = torch.from_numpy(b.out_init).to(cuda)
    fidx = torch.from_numpy(b.fac_index[:, None] * b.d + np.arange(b.d)[None, :]).to(cuda)
    forward_indexed(b.d, b.n, b.stride, fac, fidx, x, y, torch.from_numpy(out_map).to(cuda),
                    input_index=torch.from_numpy(in_map).to(cuda))
    torch.cuda.synchronize()
    assert O.rel_l2(y.cpu().numpy(), O.forward(b2)) <= 1e-13


def test_indexed_rejects_small_scratch(cuda):
    import kronmult_gb300 as K
    from kronmult_gb300 import _lib

    lib = _lib.lib()
    dummy = 256
    rc = lib.kronmult_indexed_f64_async(3, 4, 4, dummy, 16, dummy, dummy, 64, None, dummy, 64, dummy, 10, dummy,
                                        8, None)
    assert rc == 1
    assert lib.kronmult_indexed_scratch_bytes(3, 10) == 10 * 5 * 8


def test_indexed_graph_capture(cuda):
    """The indexed forward (table expansion + forward) captured in a CUDA graph and
    replayed twice adds the product twice."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import forward_indexed

    b = W.config5(scale=16 / 2048)
    fac = torch.from_numpy(b.factors).to(cuda)
    x = torch.from_numpy(b.inputs).to(cuda)
    y = torch.zeros((b.n_out, b.N), dtype=torch.float64, device=cuda)
    fidx = torch.from_numpy(b.fac_index[:, None] * b.d + np.arange(b.d)[None, :]).to(cuda).to(torch.int32)
    oidx = torch.from_numpy(b.out_index).to(cuda).to(torch.int32)
    st = torch.cuda.Stream(cuda)
    with torch.cuda.stream(st):
        scratch = forward_indexed(b.d, b.n, b.stride, fac, fidx, x, y, oidx, stream=st)  # warm-up, plans
    torch.cuda.synchronize()
    y.zero_()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st):
        forward_indexed(b.d, b.n, b.stride, fac, fidx, x, y, oidx, scratch=scratch, stream=st)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    want = 2 * (O.forward(b) - b.out_init)
    assert O.rel_l2(y.cpu().numpy(), want) <= 1e-13
