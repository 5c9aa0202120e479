"""Runs the reference's own GPU kernel (kronmult_gpu/kronmult.cu) on the current GPU.

TEST INFRASTRUCTURE ONLY: the comparator for tests/ and bench.py's report.  The
kernel is compiled unmodified from the reference sources into _ref/kronmult_gpu_ref.cubin
by oracle/Makefile (ref_gpu_shim.cu); this module loads that cubin with the CUDA
driver API and launches `cuda_kronmult_batchelement<T>` exactly as the reference's
host code does (kronmult_gpu/kronmult.cu:173-197): one CTA per entry, min(1024, n^d)
threads, no dynamic shared memory.

Like the reference, the kernel overwrites `input` and `workspace`
(kronmult_gpu/kronmult.cu:119-121), and it allocates its transpose scratch with
device-side `new` (kronmult_gpu/kronmult.cu:156).  The float kernel has a
`__syncthreads()` inside a loop (kronmult_gpu/kronmult.cu:74) that diverges when
n^d > 1024 and n^d is not a multiple of 1024; such shapes are refused here rather
than run.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "kronmult_gpu_ref.cubin")
SYMBOLS = os.path.join(HERE, "_ref", "kronmult_gpu_ref.symbols")

_state: dict = {}


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(SYMBOLS)


def _cuda():
    if "cuda" not in _state:
        lib = ctypes.CDLL("libcuda.so.1")
        for name in ("cuInit", "cuCtxGetCurrent", "cuModuleLoad", "cuModuleGetFunction", "cuLaunchKernel",
                     "cuCtxSetLimit", "cuGetErrorString"):
            getattr(lib, name).restype = ctypes.c_int
        _state["cuda"] = lib
    return _state["cuda"]


def _check(rc: int, what: str) -> None:
    if rc != 0:
        s = ctypes.c_char_p()
        _cuda().cuGetErrorString(rc, ctypes.byref(s))
        raise RuntimeError(f"{what} failed: {rc} {s.value.decode() if s.value else ''}")


def _kernel(dtype: str):
    """Function handle of cuda_kronmult_batchelement<double|float> (dtype 'f64'/'f32')."""
    key = ("fn", dtype)
    if key in _state:
        return _state[key]
    if not available():
        raise FileNotFoundError("reference cubin not built (oracle/Makefile needs the reference sources)")
    import torch

    torch.cuda.init()
    torch.zeros(1, device="cuda")  # make the primary context current in this thread
    cu = _cuda()
    _check(cu.cuInit(0), "cuInit")
    if "module" not in _state:
        # generous device heap for the kernel's per-CTA `new` (8 MB by default)
        cu.cuCtxSetLimit(ctypes.c_int(2), ctypes.c_size_t(64 << 20))  # CU_LIMIT_MALLOC_HEAP_SIZE
        mod = ctypes.c_void_p()
        _check(cu.cuModuleLoad(ctypes.byref(mod), CUBIN.encode()), "cuModuleLoad")
        _state["module"] = mod
    tag = "Id" if dtype == "f64" else "If"
    names = [ln.strip() for ln in open(SYMBOLS)]
    pat = re.compile(r"^_Z26cuda_kronmult_batchelement" + tag + r"EviiPKPKT_iPPS0_iS6_S6_i$")
    name = next(n for n in names if pat.match(n))
    fn = ctypes.c_void_p()
    _check(cu.cuModuleGetFunction(ctypes.byref(fn), _state["module"], name.encode()), "cuModuleGetFunction")
    _state[key] = fn
    return fn


def launch(d: int, n: int, mats_ptr: int, stride: int, in_ptr: int, out_ptr: int, ws_ptr: int, nb: int,
           dtype: str = "f64", stream: int = 0) -> None:
    """Enqueue the reference kernel on `stream` with device pointer tables (as the reference's
    kronmult_batched<T> would, minus its final cudaDeviceSynchronize)."""
    N = n ** d
    if nb <= 0 or N <= 0:
        return
    block = min(1024, N)
    if dtype == "f32" and N > 1024 and N % 1024 != 0:
        raise ValueError("the reference float kernel would reach a divergent __syncthreads for this n^d")
    fn = _kernel(dtype)
    args = [ctypes.c_int(d), ctypes.c_int(n), ctypes.c_void_p(mats_ptr), ctypes.c_int(stride),
            ctypes.c_void_p(in_ptr), ctypes.c_int(N), ctypes.c_void_p(out_ptr), ctypes.c_void_p(ws_ptr),
            ctypes.c_int(nb)]
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
    _check(_cuda().cuLaunchKernel(fn, nb, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream), params, None),
           "cuLaunchKernel")
