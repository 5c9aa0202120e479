"""Generate the golden fixtures under tests/golden/ from the reference's own code.

Each fixture is a small seeded batch (factors, inputs, initial outputs, index
maps) together with the output that the reference's CPU library, kronmult_omp,
produces for it.  kronmult_omp is compiled unmodified from the reference sources
by oracle/Makefile into oracle/_ref/; this script therefore runs only where those
sources exist.  The fixtures are committed so that the tests on any machine pin
both the C oracle and the CUDA library to the reference's outputs.

Run:  make -C oracle && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from kronmult_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def reference_style_aliasing(nb: int, distinct: int) -> np.ndarray:
    """Output map of the reference tests: entry i < distinct -> i, else (i*distinct)//nb
    (tests/utils/utils_cpu.h:73-83); not contiguous."""
    idx = np.arange(nb, dtype=np.int64)
    return np.where(idx < distinct, idx, (idx * distinct) // nb)


def with_out_index(b: W.Batch, out_index: np.ndarray, n_out: int, seed: int) -> W.Batch:
    rng = np.random.Generator(np.random.PCG64(seed))
    return W.Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs,
                   rng.standard_normal((n_out, b.N)), b.fac_index, out_index.astype(np.int64), dict(b.meta))


def cases():
    out = []
    # reference test shapes: toy (n=4, d=1) and small (n=4, d=2), stride 67, 5 distinct outputs
    # reached through the reference's non-contiguous aliasing pattern
    for name, d, n, nb in (("toy", 1, 4, 8), ("small", 2, 4, 64)):
        b = W.make_batch(d, n, 67, nb, 1, seed=7 + d, name=name)
        out.append(with_out_index(b, reference_style_aliasing(nb, 5), 5, seed=70 + d))
    out.append(W.config1(scale=32 / 1024))                           # C1 shape, 32 outputs x 8
    b = W.config2(scale=1 / 4096)                                     # C2 shape, 1 output x 9
    out.append(b)
    for b in W.config3(scale=0.0):                                    # C3 group shapes, 1 output each
        out.append(b)
    rng = np.random.Generator(np.random.PCG64(11))
    out.append(W.make_batch(4, 8, 8, 1, 8, seed=1104, name="c4_small", factor_scale=1 / 8))
    out.append(W.make_batch(3, 6, 6, 4, 8, seed=1105, name="c5_small", shared_factors=True))
    # edge cases
    out.append(W.make_batch(3, 1, 1, 3, 2, seed=21, name="n1_d3"))
    out.append(W.make_batch(3, 3, 5, 4, 3, seed=22, name="n3_d3_stride5", out_init="normal"))
    out.append(W.make_batch(2, 5, 9, 3, 4, seed=23, name="n5_d2_stride9"))
    out.append(W.make_batch(2, 7, 7, 2, 5, seed=24, name="n7_d2"))
    out.append(W.make_batch(10, 2, 3, 2, 3, seed=25, name="n2_d10"))
    out.append(W.make_batch(1, 8, 8, 3, 3, seed=26, name="n8_d1"))
    out.append(W.make_batch(2, 9, 11, 2, 3, seed=27, name="n9_d2_generic"))
    out.append(W.make_batch(2, 16, 16, 2, 2, seed=28, name="n16_d2_generic"))
    b = W.make_batch(2, 4, 4, 6, 5, seed=29, name="random_aliasing")
    out.append(with_out_index(b, rng.integers(0, 6, size=b.nb), 6, seed=290))
    out.append(W.make_batch(2, 4, 4, 0, 1, seed=30, name="empty_batch"))
    return out


def main():
    assert O.available("reference"), "build oracle/_ref first: make -C oracle"
    manifest = {}
    for b in cases():
        entry = {"d": b.d, "n": b.n, "stride": b.stride, "nb": b.nb, "n_out": b.n_out}
        arrays = dict(d=b.d, n=b.n, stride=b.stride, block=b.block, factors=b.factors, inputs=b.inputs,
                      out_init=b.out_init, fac_index=b.fac_index, out_index=b.out_index)
        # one OpenMP thread: the reference's atomic additions then happen in entry order
        arrays["expected_f64"] = O.forward(b, impl="reference", nthreads=1)
        arrays["expected_f32"] = O.forward(b, dtype=np.float32, impl="reference", nthreads=1)
        if b.name == "c5_small":
            # adjoint golden: grad_input[k] = kron(A_k^T) . grad_out[out(k)], i.e. the reference
            # applied with transposed factor copies to the gathered output gradients
            g = np.random.Generator(np.random.PCG64(1106)).standard_normal((b.n_out, b.N))
            fac_t = np.zeros((b.factors.shape[0], b.n * b.n))
            for r in range(b.factors.shape[0]):
                A = b.factors[r].reshape(-1)
                M = np.array([[A[rr + kk * b.stride] for kk in range(b.n)] for rr in range(b.n)])
                fac_t[r] = M.T.reshape(-1, order="F")
            bt = W.Batch("c5_adjoint", b.d, b.n, b.n, b.n * b.n, fac_t, g[b.out_index], np.zeros((b.nb, b.N)),
                         b.fac_index, np.arange(b.nb, dtype=np.int64))
            arrays["grad_out"] = g
            arrays["expected_grad_input_f64"] = O.forward(bt, impl="reference", nthreads=1)
        np.savez_compressed(os.path.join(HERE, f"{b.name}.npz"), **arrays)
        manifest[b.name] = entry
        print(f"{b.name:24s} d={b.d} n={b.n} stride={b.stride} nb={b.nb} outputs={b.n_out}")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "kronmult_omp built by oracle/Makefile (ref_omp_shim.cpp), OMP_NUM_THREADS=1",
                   "cases": manifest}, f, indent=1)


if __name__ == "__main__":
    main()
