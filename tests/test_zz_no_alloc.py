"""The allocation-free forward, kronmult_batched_f64_noalloc, for callers that
cannot allocate device memory where they run the product (application-owned
memory pools, allocator-free callbacks).  It keeps its work list in a fixed array
inside the library; these tests call it through the C ABI and compare it with the
regular entry point, kronmult_batched_f64_async, on two calls in a row.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

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


@pytest.mark.parametrize("shape", ["d6_n4_stride8_fan9", "d3_n4_fan8", "d3_n6_ragged"])
def test_noalloc_matches_regular_entry_point_twice(shape):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kronmult_gb300 import DeviceBatch, _lib
    from kronmult_gb300 import workloads as W

    lib = _lib.lib()
    if shape == "d6_n4_stride8_fan9":
        b = W.config2(scale=96 / 4096)
    elif shape == "d3_n4_fan8":
        b = W.config1(scale=64 / 1024)
    else:
        b = W.make_batch(3, 6, 7, 40, np.random.Generator(np.random.PCG64(3)).integers(1, 28, 40), seed=4)
    db = DeviceBatch.from_host(b, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream

    db.outputs.zero_()
    assert _regular(lib, db, stream) == 0
    torch.cuda.synchronize()
    want = db.outputs.clone()

    results = []
    for _ in range(2):  # two calls in a row: the shared array keeps the last call's contents
        db.outputs.zero_()
        assert _noalloc(lib, db, stream) == 0
        torch.cuda.synchronize()
        results.append(db.outputs.clone())
    for got in results:
        assert _rel(got, want) <= TOL64
    # every output's entries form one contiguous run here: one addition per element
    assert torch.equal(results[0], results[1])


def test_noalloc_rejects_batches_beyond_its_array():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kronmult_gb300 import _lib

    lib = _lib.lib()
    dummy = ctypes.c_void_p(256)
    rc = lib.kronmult_batched_f64_noalloc(3, 4, dummy, 4, dummy, dummy, _lib.KRONMULT_NOALLOC_MAX_ENTRIES + 1, None)
    assert rc == 1  # cudaErrorInvalidValue, nothing launched
