"""ctypes binding of libkronmult_gb300.so (C ABI: include/kronmult_gb300.h).

The library is the product: there is no CPU fallback.  If the shared library
has not been built, loading raises instead of silently computing elsewhere.
"""
from __future__ import annotations

import ctypes
import os
import threading

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libkronmult_gb300.so")

KRONMULT_COMPUTE_FP32 = 0
KRONMULT_COMPUTE_TF32 = 1
KRONMULT_COMPUTE_BF16 = 2
KRONMULT_COMPUTE_BF16X3 = 3


class Tuning(ctypes.Structure):
    """Mirror of `kronmult_tuning`: launch-shape override, zero = heuristic."""

    _fields_ = [("team_size", ctypes.c_int), ("ctas_per_sm", ctypes.c_int), ("entries_per_team", ctypes.c_int),
                ("prefetch", ctypes.c_int), ("fp64_path", ctypes.c_int)]


class Group(ctypes.Structure):
    """Mirror of `kronmult_group`: one group's arguments (device pointer tables)."""

    _fields_ = [("matrix_count", ctypes.c_int), ("matrix_size", ctypes.c_int), ("matrix_stride", ctypes.c_int),
                ("nb_batch", ctypes.c_int), ("matrix_list_batched", ctypes.c_void_p),
                ("input_batched", ctypes.c_void_p), ("output_batched", ctypes.c_void_p)]


class AdjointGroup(ctypes.Structure):
    """Mirror of `kronmult_adjoint_group`: one adjoint group's arguments."""

    _fields_ = [("matrix_count", ctypes.c_int), ("matrix_size", ctypes.c_int), ("matrix_stride", ctypes.c_int),
                ("nb_batch", ctypes.c_int), ("matrix_list_batched", ctypes.c_void_p),
                ("input_batched", ctypes.c_void_p), ("grad_output_batched", ctypes.c_void_p),
                ("grad_input_batched", ctypes.c_void_p), ("grad_matrix_list_batched", ctypes.c_void_p),
                ("grad_matrix_stride", ctypes.c_int)]


KRONMULT_DTYPE_F64 = 0
KRONMULT_DTYPE_F32 = 1
KRONMULT_DTYPE_F32_F64OUT = 2
KRONMULT_DTYPE_F64_EMULATED = 3
KRONMULT_MODE_ATOMIC = 0
KRONMULT_MODE_DETERMINISTIC = 1
KRONMULT_NOALLOC_MAX_ENTRIES = 1048576


class KronmultError(RuntimeError):
    """A non-zero status (a cudaError_t value) returned by the library."""

    def __init__(self, status: int, where: str, detail: str | None = None):
        self.status = status
        super().__init__(f"{where} failed with status {status}: {detail or error_string(status)}")


_lock = threading.Lock()
_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_TP = ctypes.POINTER(Tuning)

# (name, restype, argtypes); every symbol include/kronmult_gb300.h declares
SIGNATURES = {
    "kronmult_batched_f64": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i]),
    "kronmult_batched_f32": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i]),
    "kronmult_batched_f64_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _vp, _TP]),
    "kronmult_batched_f32_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _vp, _TP]),
    "kronmult_batched_f32_f64out_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _vp, _TP]),
    "kronmult_batched_adjoint_f64_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _TP]),
    "kronmult_batched_adjoint_f32_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _TP]),
    "kronmult_grouped_plan_create": (_i, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Group), _i, _i, _i,
                                         _TP]),
    "kronmult_grouped_plan_create_with_adjoint": (_i, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Group), _i,
                                                      ctypes.POINTER(AdjointGroup), _i, _i, _i, _TP]),
    "kronmult_grouped_run": (_i, [_vp, _vp]),
    "kronmult_grouped_regroup": (_i, [_vp, _vp]),
    "kronmult_grouped_plan_info": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong), _i]),
    "kronmult_grouped_plan_destroy": (_i, [_vp]),
    "kronmult_autotune_forward": (_i, [_i, _i, _i, _i, _TP, ctypes.POINTER(ctypes.c_float)]),
    "kronmult_tuning_cache_get": (_i, [_i, _i, _i, _TP]),
    "kronmult_tuning_cache_set": (_i, [_i, _i, _i, _TP]),
    "kronmult_tuning_cache_clear": (_i, []),
    "kronmult_tuning_cache_save": (_i, [ctypes.c_char_p]),
    "kronmult_tuning_cache_load": (_i, [ctypes.c_char_p]),
    "kronmult_device_error": (_i, [ctypes.POINTER(ctypes.c_int), _i]),
    "kronmult_diag_wait_selftest": (_i, [ctypes.POINTER(ctypes.c_int)]),
    "kronmult_indexed_scratch_bytes": (ctypes.c_longlong, [_i, _i]),
    "kronmult_host_device_pointer": (_i, [_vp, ctypes.POINTER(ctypes.c_void_p)]),
    "kronmult_indexed_f64_async": (_i, [_i, _i, _i, _vp, ctypes.c_longlong, _vp, _vp, ctypes.c_longlong, _vp, _vp,
                                        ctypes.c_longlong, _vp, _i, _vp, ctypes.c_longlong, _vp]),
    "kronmult_indexed_f32_async": (_i, [_i, _i, _i, _vp, ctypes.c_longlong, _vp, _vp, ctypes.c_longlong, _vp, _vp,
                                        ctypes.c_longlong, _vp, _i, _vp, ctypes.c_longlong, _vp]),
    "kronmult_batched_f64_emulated_async": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _vp]),
    "kronmult_batched_f64_noalloc": (_i, [_i, _i, _vp, _i, _vp, _vp, _i, _vp]),
    "kronmult_diag_fp64_fma_gflops": (_i, [ctypes.POINTER(ctypes.c_double)]),
    "kronmult_diag_fp64_mma_gflops": (_i, [ctypes.POINTER(ctypes.c_double)]),
    "kronmult_diag_int8_mma_tops": (_i, [ctypes.POINTER(ctypes.c_double)]),
    "kronmult_diag_ozaki_elementwise_ms": (_i, [ctypes.c_longlong, _i, ctypes.POINTER(ctypes.c_double)]),
    "kronmult_diag_fp64_mma_rounding": (_i, [ctypes.POINTER(ctypes.c_ulonglong)]),
    "kronmult_diag_fp64_pipe_share": (_i, [ctypes.POINTER(ctypes.c_double)]),
    "kronmult_pow_int": (ctypes.c_longlong, [_i, _i]),
    "kronmult_error_string": (ctypes.c_char_p, [_i]),
    "kronmult_abi_version": (_i, []),
}


def lib() -> ctypes.CDLL:
    """Load the library once; raise if it is missing (build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build the CUDA library first "
                    "(python -c 'import __graft_entry__ as g; g.build()')")
            h = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(h, name)
                fn.restype = res
                fn.argtypes = args
            _lib = h
    return _lib


def error_string(status: int) -> str:
    try:
        s = lib().kronmult_error_string(int(status))
        return s.decode() if s else "unknown"
    except Exception:  # pragma: no cover - only used while formatting another error
        return "unknown"


def check(status: int, where: str) -> None:
    if status != 0:
        raise KronmultError(status, where)


def tuning_ptr(t: Tuning | dict | None):
    if t is None:
        return None
    if isinstance(t, dict):
        t = Tuning(int(t.get("team_size", 0)), int(t.get("ctas_per_sm", 0)), int(t.get("entries_per_team", 0)),
                   int(t.get("prefetch", 0)), int(t.get("fp64_path", 0)))
    return ctypes.byref(t)
