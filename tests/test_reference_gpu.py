"""Parity with the reference's own GPU kernel (kronmult_gpu/kronmult.cu built for
sm_103a from the reference sources, run through oracle/ref_gpu.py) on the same
inputs.  Per entry the arithmetic is the same k-ascending FMA chain, so with one
output per entry the results are bitwise identical; with shared outputs only the
order of the atomic additions differs."""
import numpy as np
import pytest
import torch

from oracle import ref_gpu

pytestmark = pytest.mark.gpu


def reference_run(db, dtype="f64"):
    """The reference kernel on copies of the inputs (it overwrites inputs and workspaces)."""
    x = db.inputs.clone()
    ws = torch.empty_like(x)
    out = db.outputs.clone()
    es = x.element_size()
    k = torch.arange(db.nb, device=x.device, dtype=torch.int64)
    in_ptrs = x.data_ptr() + k * (db.N * es)
    ws_ptrs = ws.data_ptr() + k * (db.N * es)
    out_ptrs = out.data_ptr() + db.out_index * (out.shape[1] * es)
    torch.cuda.synchronize()
    ref_gpu.launch(db.d, db.n, db.mat_ptrs.data_ptr(), db.stride, in_ptrs.data_ptr(), out_ptrs.data_ptr(),
                   ws_ptrs.data_ptr(), db.nb, dtype=dtype)
    torch.cuda.synchronize()
    return out


def needs_ref():
    if not ref_gpu.available():
        pytest.skip("reference cubin not built (the reference sources are needed to build it)")


@pytest.mark.parametrize("d,n,stride", [(3, 4, 4), (6, 4, 8), (3, 6, 6), (2, 8, 8), (6, 3, 5), (4, 4, 67)])
def test_bitwise_per_entry_f64(cuda, d, n, stride):
    needs_ref()
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, stride, 40, 1, seed=600 + d * 10 + n)  # one output per entry
    db = DeviceBatch.from_host(b, device=cuda)
    want = reference_run(db)
    db.forward(sync=True)
    assert torch.equal(db.outputs, want)


@pytest.mark.parametrize("d,n,stride,dtype", [(5, 8, 8, torch.float64), (10, 3, 4, torch.float64),
                                              (5, 8, 8, torch.float32), (6, 8, 67, torch.float64)])
def test_bitwise_per_entry_large(cuda, d, n, stride, dtype):
    """Vectors beyond shared memory (two passes through the workspace) against the
    reference kernel's one-vector sweep: identical bits per entry."""
    needs_ref()
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    nb = 3 if n ** d > 100000 else 12
    b = W.make_batch(d, n, stride, nb, 1, seed=660 + d * 10 + n)
    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype, with_workspace=True)
    want = reference_run(db, "f64" if dtype == torch.float64 else "f32")
    db.forward(sync=True)
    assert torch.equal(db.outputs, want)


@pytest.mark.parametrize("d,n,stride", [(6, 4, 8), (4, 8, 8), (3, 8, 11)])
def test_bitwise_per_entry_f32(cuda, d, n, stride):
    """FP32 two-modes-per-pass kernels (n = 4; n = 8 with a lane pair per bi-fibre)
    against the reference float kernel: identical bits per entry."""
    needs_ref()
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, stride, 40, 1, seed=650 + d, block=n * stride)
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32)
    want = reference_run(db, "f32")
    db.forward(sync=True)
    assert torch.equal(db.outputs, want)


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_shared_outputs_vs_reference_kernel(cuda, cfg):
    needs_ref()
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.config1() if cfg == "c1" else W.config2(scale=128 / 4096)
    db = DeviceBatch.from_host(b, device=cuda)
    want = reference_run(db)
    db.forward(sync=True)
    err = (torch.linalg.norm(db.outputs - want) / torch.linalg.norm(want)).item()
    assert err <= 1e-13


@pytest.mark.parametrize("seed", list(range(16)))
def test_bitwise_random_shapes(cuda, seed):
    """Seeded random shapes (n = 1..10, strides beyond n, one output per entry): our
    forward and the reference kernel agree bit for bit in FP64, and in FP32 where the
    reference float kernel is well defined (N <= 1024 or a multiple of 1024)."""
    needs_ref()
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(9100 + seed))
    n = int(rng.integers(1, 11))
    max_d = max(1, int(np.floor(np.log(20000) / np.log(max(n, 2)))))
    d = int(rng.integers(1, min(max_d, 7) + 1))
    stride = n + int(rng.integers(0, 3))
    nb = int(rng.integers(1, 40))
    b = W.make_batch(d, n, stride, nb, 1, seed=9200 + seed)
    for dtype, tag in ((torch.float64, "f64"), (torch.float32, "f32")):
        N = n ** d
        if tag == "f32" and N > 1024 and N % 1024:
            continue
        db = DeviceBatch.from_host(b, device=cuda, dtype=dtype, with_workspace=True)
        want = reference_run(db, tag)
        db.forward(sync=True)
        assert torch.equal(db.outputs, want), (d, n, stride, nb, tag)
