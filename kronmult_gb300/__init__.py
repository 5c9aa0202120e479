"""kronmult_gb300: batched Kronecker-product matrix-vector product for GB300 (sm_103a).

For every entry k: output[k] += kron(A_{k,0}, ..., A_{k,d-1}) . input[k], as the
reference's `kronmult_batched` (kronmult_gpu/kronmult.cuh:28-32).  The compute
runs in the hand-written CUDA library libkronmult_gb300.so behind a C ABI
(include/kronmult_gb300.h); this package is its Python host mirror.
"""
from ._lib import (KRONMULT_COMPUTE_BF16, KRONMULT_COMPUTE_BF16X3, KRONMULT_COMPUTE_FP32, KRONMULT_COMPUTE_TF32,
                   KronmultError, Tuning, lib)
from .api import (DeviceBatch, adjoint, check_device_error, forward_f32_f64out, kronmult_batched,
                  kronmult_batched_async)
from .workloads import Batch, make_batch

__all__ = [
    "Batch", "DeviceBatch", "adjoint", "KronmultError", "Tuning", "lib", "make_batch", "kronmult_batched",
    "kronmult_batched_async", "forward_f32_f64out", "check_device_error", "KRONMULT_COMPUTE_FP32", "KRONMULT_COMPUTE_TF32",
    "KRONMULT_COMPUTE_BF16", "KRONMULT_COMPUTE_BF16X3",
]
