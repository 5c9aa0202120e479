"""Python front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline / reference legs, never by the kronmult_gb300 package.

Three implementations of the same maths, all on host arrays of a
`kronmult_gb300.workloads.Batch`:
  port       liboracle.so, the C restatement in kronmult_oracle.c
             (kronmult_omp/kronmult.hpp:32-104 and linear_algebra.hpp:78-121)
  reference  _ref/libkronmult_omp_ref.so, the reference's own kronmult_omp built from
             its sources by oracle/Makefile (only where those sources exist)
  naive      the explicit-Kronecker check of tests/utils/kronmult_naive.h:73-121,
             restated in kronmult_oracle.c (small n^d only)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libkronmult_omp_ref.so")

_libs: dict[str, ctypes.CDLL] = {}


def build(ref: bool = True) -> None:
    """Build liboracle.so (and _ref/ when the reference sources are present) with make."""
    targets = ["all"] if ref else ["liboracle.so"]
    subprocess.run(["make", "-s", "-C", HERE, *targets], check=True)


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind in ("port", "naive") else REF_LIB)


def _load(kind: str) -> ctypes.CDLL:
    key = "reference" if kind == "reference" else "port"
    if key in _libs:
        return _libs[key]
    path = REF_LIB if key == "reference" else PORT_LIB
    if not os.path.exists(path):
        if key == "port":
            build(ref=False)
        else:
            raise FileNotFoundError(f"{path} not built (the reference sources are needed to build it)")
    h = ctypes.CDLL(path)
    vp, i = ctypes.c_void_p, ctypes.c_int
    if key == "port":
        for suf in ("f64", "f32"):
            f = getattr(h, f"oracle_kronmult_batched_{suf}")
            f.restype, f.argtypes = i, [i, i, vp, i, vp, vp, i, i]
            f = getattr(h, f"oracle_kronmult_naive_{suf}")
            f.restype, f.argtypes = i, [i, i, vp, i, vp, vp]
        h.oracle_max_threads.restype = i
    else:
        for suf in ("f64", "f32"):
            f = getattr(h, f"ref_kronmult_batched_{suf}")
            f.restype, f.argtypes = i, [i, i, vp, i, vp, vp, vp, i]
            f = getattr(h, f"ref_kronmult_naive_{suf}")
            f.restype, f.argtypes = i, [i, i, vp, i, vp, vp, i]
        h.ref_max_threads.restype = i
        h.ref_set_num_threads.restype, h.ref_set_num_threads.argtypes = None, [i]
    _libs[key] = h
    return h


def max_threads(kind: str = "port") -> int:
    h = _load(kind)
    return h.oracle_max_threads() if kind != "reference" else h.ref_max_threads()


def _pointer_tables(b, factors, inputs, outs):
    fes = factors.itemsize
    d = b.d
    i = np.arange(d, dtype=np.uint64)
    mats = (np.uint64(factors.ctypes.data)
            + ((b.fac_index.astype(np.uint64)[:, None] * np.uint64(d) + i[None, :])
               * np.uint64(factors.shape[1] * fes))).reshape(-1)
    k = np.arange(b.nb, dtype=np.uint64)
    ins = np.uint64(inputs.ctypes.data) + k * np.uint64(inputs.shape[1] * inputs.itemsize)
    outp = np.uint64(outs.ctypes.data) + b.out_index.astype(np.uint64) * np.uint64(outs.shape[1] * outs.itemsize)
    return np.ascontiguousarray(mats), np.ascontiguousarray(ins), np.ascontiguousarray(outp)


def forward(b, dtype=np.float64, impl: str = "port", nthreads: int = 0, out_dtype=None) -> np.ndarray:
    """Return out_init + sum over entries of kron(A_k) . x_k as an (E, N) array.

    `dtype` is the storage/compute type of factors and inputs; `out_dtype` (default:
    dtype) the type of the output accumulation.  A float32 compute with a float64
    output is evaluated as the float32 sweep per entry followed by a float64 sum.
    """
    dt = np.dtype(dtype)
    odt = np.dtype(out_dtype) if out_dtype is not None else dt
    suf = "f64" if dt == np.float64 else "f32"
    factors = np.ascontiguousarray(b.factors, dtype=dt)
    inputs = np.ascontiguousarray(b.inputs, dtype=dt)
    if odt != dt:
        # per-entry products in dt, accumulated in odt
        outs = np.zeros((b.nb, b.N), dtype=dt)
        one = np.arange(b.nb, dtype=np.int64)
        proxy = _Proxy(b, out_index=one)
        mats, ins, outp = _pointer_tables(proxy, factors, inputs, outs)
        _call(impl, suf, b, mats, ins, outp, inputs, nthreads)
        res = np.array(b.out_init, dtype=odt, copy=True)
        np.add.at(res, b.out_index, outs.astype(odt))
        return res
    outs = np.array(b.out_init, dtype=dt, copy=True)
    mats, ins, outp = _pointer_tables(b, factors, inputs, outs)
    _call(impl, suf, b, mats, ins, outp, inputs, nthreads)
    return outs


class _Proxy:
    def __init__(self, b, out_index):
        self.d, self.nb, self.fac_index, self.out_index = b.d, b.nb, b.fac_index, out_index


def _call(impl, suf, b, mats, ins, outp, inputs, nthreads):
    if b.nb == 0:
        return
    if impl == "port":
        h = _load("port")
        rc = getattr(h, f"oracle_kronmult_batched_{suf}")(b.d, b.n, mats.ctypes.data, b.stride, ins.ctypes.data,
                                                          outp.ctypes.data, b.nb, int(nthreads))
    elif impl == "reference":
        h = _load("reference")
        # the reference clobbers inputs and workspaces: give it copies
        icopy = inputs.copy()
        ws = np.empty_like(icopy)
        k = np.arange(b.nb, dtype=np.uint64)
        ins2 = np.uint64(icopy.ctypes.data) + k * np.uint64(icopy.shape[1] * icopy.itemsize)
        wsp = np.uint64(ws.ctypes.data) + k * np.uint64(ws.shape[1] * ws.itemsize)
        if nthreads:
            h.ref_set_num_threads(int(nthreads))
        rc = getattr(h, f"ref_kronmult_batched_{suf}")(b.d, b.n, mats.ctypes.data, b.stride, ins2.ctypes.data,
                                                       outp.ctypes.data, wsp.ctypes.data, b.nb)
    elif impl == "naive":
        h = _load("port")
        f = getattr(h, f"oracle_kronmult_naive_{suf}")
        rc = 0
        esz = inputs.itemsize
        for k in range(b.nb):
            m = mats[k * b.d:(k + 1) * b.d]
            rc |= f(b.d, b.n, m.ctypes.data, b.stride, int(ins[k]), int(outp[k]))
    elif impl == "reference_naive":
        h = _load("reference")
        rc = getattr(h, f"ref_kronmult_naive_{suf}")(b.d, b.n, mats.ctypes.data, b.stride, ins.ctypes.data,
                                                     outp.ctypes.data, b.nb)
    else:
        raise ValueError(f"unknown oracle implementation {impl!r}")
    if rc != 0:
        raise RuntimeError(f"oracle {impl} failed with status {rc}")


def factor_matrices(b, dtype=np.float64) -> np.ndarray:
    """Every factor row of the batch as an (rows, n, n) array of n x n matrices
    (row r, column c at offset r + c*stride of the col-major storage)."""
    n, st = b.n, b.stride
    F = np.asarray(b.factors, dtype=dtype)[:, :n * st].reshape(-1, n, st)[:, :, :n]  # [row, c, r]
    return np.ascontiguousarray(F.transpose(0, 2, 1))


def transposed_batch(b, grad_out):
    """The batch whose forward is the adjoint's grad_input: factors A^T (stride n), each
    entry's input the gradient of the output it adds into, one output per entry.  The
    adjoint of kronmult_batched is the reference applied with transposed factors
    (kronmult_omp/kronmult.hpp:77-104 on A_i^T)."""
    from kronmult_gb300.workloads import Batch

    n = b.n
    At = factor_matrices(b).transpose(0, 2, 1)  # A^T per row
    fac_t = np.ascontiguousarray(At.transpose(0, 2, 1)).reshape(-1, n * n)  # col-major, ld n
    return Batch(b.name + "_T", b.d, n, n, n * n, fac_t, np.asarray(grad_out)[b.out_index],
                 np.zeros((b.nb, b.N)), b.fac_index, np.arange(b.nb, dtype=np.int64))


def _apply_mode(T, A, axis):
    """T (B, n, ..., n) with the batch's matrices A (B, n, n) applied along tensor axis `axis`."""
    Tm = np.moveaxis(T, axis + 1, -1)
    sh = Tm.shape
    R = np.matmul(Tm.reshape(sh[0], -1, sh[-1]), A.transpose(0, 2, 1)).reshape(sh)
    return np.moveaxis(R, -1, axis + 1)


def grad_factors(b, grad_out, dtype=np.float64) -> np.ndarray:
    """dL/dA for L = sum_e <grad_out[e], out[e]>, as (rows, n, n) matrices summed over the
    entries sharing a factor row.  Mode-unfolding formula: for entry k and mode i,
    dL/dA_{k,i} = G_(i) . U_(i)^T, with G the gradient of entry k's output as an n^d tensor
    (A_0 the most significant index) and U the input with every factor but A_i applied.
    The reference has no gradient; this formula is checked against central finite
    differences of the forward in the tests."""
    n, d = b.n, b.d
    A = factor_matrices(b, dtype)
    rows = A.shape[0]
    X = np.asarray(b.inputs, dtype=dtype).reshape((b.nb,) + (n,) * d)
    G = np.asarray(grad_out, dtype=dtype)[b.out_index].reshape((b.nb,) + (n,) * d)
    out = np.zeros((rows, n, n), dtype=dtype)
    for i in range(d):
        U = X
        for m in range(d):
            if m != i:
                U = _apply_mode(U, A[b.fac_index * d + m], m)
        Gi = np.moveaxis(G, i + 1, 1).reshape(b.nb, n, -1)
        Ui = np.moveaxis(U, i + 1, 1).reshape(b.nb, n, -1)
        np.add.at(out, b.fac_index * d + i, np.matmul(Gi, Ui.transpose(0, 2, 1)))
    return out


def rel_l2(a, b) -> float:
    """||a - b||_2 / ||b||_2 over all elements (b is the reference)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)


def max_rel(a, b, eps: float = 1e-300) -> float:
    """max |a - b| / max |b| (normwise maximum error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / max(den, eps)) if a.size else 0.0
