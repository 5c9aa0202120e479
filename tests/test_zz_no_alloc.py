"""The allocation-free forward, kronmult_batched_f64_noalloc, for callers that
cannot allocate device memory where they run the product (application-owned
memory pools, allocator-free callbacks).  It keeps its work list in a fixed array
inside the library; these tests call it through the C ABI, two calls in a row, and
compare it with the regular entry point, kronmult_batched_f64_async, and with the
oracle (a restatement of the reference's kronmult_omp) on the same inputs.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-13


def _noalloc(lib, db, stream):
    return lib.kronmult_batched_f64_noalloc(db.d, db.n, db.mat_ptrs.data_ptr(), db.stride, db.in_ptrs.data_ptr(),
                                            db.out_ptrs.data_ptr(), db.nb, stream)


def _regular(lib, db, stream):
    return lib.kronmult_batched_f64_async(db.d, db.n, db.mat_ptrs.data_ptr(), db.stride, db.in_ptrs.data_ptr(),
                                          db.out_ptrs.data_ptr(), None, db.nb, stream, None)


def _rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def _reference_aliasing(b, distinct):
    """The reference tests' output map (tests/utils/utils_cpu.h:79-83): entry i < distinct
    adds into output i, every other entry into output (i*distinct)//nb -- not contiguous,
    and a few long runs."""
    from kronmult_gb300.workloads import Batch

    idx = np.arange(b.nb, dtype=np.int64)
    out_index = np.where(idx < distinct, idx, (idx * distinct) // b.nb)
    return Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, b.out_init[:distinct], b.fac_index,
                 out_index)


def _batch(shape):
    from kronmult_gb300 import workloads as W

    if shape == "d6_n4_stride8_fan9":
        return W.config2(scale=96 / 4096)
    if shape == "d3_n4_fan8":
        return W.config1(scale=64 / 1024)
    if shape == "d3_n6_ragged":
        return W.make_batch(3, 6, 7, 40, np.random.Generator(np.random.PCG64(3)).integers(1, 28, 40), seed=4)
    if shape == "d4_n6_stride67_reference_aliasing_3903":
        # the reference's benchmark count (3903 entries, 5 outputs, stride 67) at n = 6, d = 4
        return _reference_aliasing(W.make_batch(4, 6, 67, 3903, 1, seed=3903, out_init="normal"), 5)
    raise ValueError(shape)


def _max_run(out_index):
    o = np.asarray(out_index)
    starts = np.flatnonzero(np.r_[True, o[1:] != o[:-1], True])
    return int(np.max(np.diff(starts))) if o.size else 0


@pytest.mark.parametrize("shape", ["d6_n4_stride8_fan9", "d3_n4_fan8", "d3_n6_ragged",
                                   "d4_n6_stride67_reference_aliasing_3903"])
def test_noalloc_matches_regular_entry_point_and_oracle_twice(shape):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kronmult_gb300 import DeviceBatch, _lib

    lib = _lib.lib()
    b = _batch(shape)
    want_oracle = O.forward(b)
    db = DeviceBatch.from_host(b, device="cuda:0")
    init = db.outputs.clone()
    stream = torch.cuda.current_stream().cuda_stream

    assert _regular(lib, db, stream) == 0
    torch.cuda.synchronize()
    want = db.outputs.clone()

    results = []
    for _ in range(2):  # two calls in a row: the shared array keeps the last call's contents
        db.outputs.copy_(init)
        assert _noalloc(lib, db, stream) == 0
        torch.cuda.synchronize()
        results.append(db.outputs.clone())
    for got in results:
        assert _rel(got, want) <= TOL64
        assert O.rel_l2(got.cpu().numpy(), want_oracle) <= TOL64
    contiguous = len(np.unique(b.out_index)) == len(np.flatnonzero(np.r_[True, np.diff(b.out_index) != 0]))
    if contiguous and _max_run(b.out_index) <= 16:
        # one addition per output element: bitwise the same on every call
        assert torch.equal(results[0], results[1])


def test_noalloc_rejects_batches_beyond_its_array():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kronmult_gb300 import _lib

    lib = _lib.lib()
    dummy = ctypes.c_void_p(256)
    rc = lib.kronmult_batched_f64_noalloc(3, 4, dummy, 4, dummy, dummy, _lib.KRONMULT_NOALLOC_MAX_ENTRIES + 1, None)
    assert rc == 1  # cudaErrorInvalidValue, nothing launched


def test_noalloc_refuses_more_than_1024_fibres():
    """n = 2, d = 12 fits shared memory (32 KB) but has 2^11 fibres: more than 4 per
    thread of a 256-thread team, cudaErrorNotSupported, nothing launched."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kronmult_gb300 import _lib

    lib = _lib.lib()
    dummy = ctypes.c_void_p(256)
    rc = lib.kronmult_batched_f64_noalloc(12, 2, dummy, 2, dummy, dummy, 4, None)
    assert rc == 801  # cudaErrorNotSupported
