"""Seeded synthetic batches with the shapes of the benchmark configurations.

A batch is described by dense host arrays plus two index maps:
  factors   (S*d, block)  factor storage; factor i of set s is row s*d+i, an
                          n x n col-major matrix with leading dimension `stride`
                          (element (r, k) at column offset r + k*stride)
  inputs    (B, N)        one input vector per entry
  out_init  (E, N)        initial value of each distinct output vector
  fac_index (B,)          factor set used by each entry
  out_index (B,)          output vector each entry adds into (entries sharing an
                          output are contiguous, as in kronmult's callers)
All values come from numpy's PCG64 generator seeded per configuration, so the
same batch is rebuilt bit-for-bit on any machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Batch:
    name: str
    d: int
    n: int
    stride: int
    block: int
    factors: np.ndarray
    inputs: np.ndarray
    out_init: np.ndarray
    fac_index: np.ndarray
    out_index: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def N(self) -> int:
        return self.n ** self.d

    @property
    def nb(self) -> int:
        return int(self.inputs.shape[0])

    @property
    def n_out(self) -> int:
        return int(self.out_init.shape[0])

    @property
    def n_sets(self) -> int:
        return int(self.factors.shape[0] // max(self.d, 1))

    def astype(self, dtype) -> "Batch":
        dt = np.dtype(dtype)
        return Batch(self.name, self.d, self.n, self.stride, self.block, self.factors.astype(dt),
                     self.inputs.astype(dt), self.out_init.astype(dt), self.fac_index, self.out_index,
                     dict(self.meta))

    def flops(self) -> float:
        """Algorithmic flops of the backward sweep: 2*d*n*N per entry."""
        return 2.0 * self.d * self.n * self.N * self.nb

    def bytes(self, in_size: int = 8, out_size: int = 8) -> float:
        """Algorithmic HBM bytes: inputs once, each distinct factor set once (n*n*d values,
        stride padding not counted), each distinct output read once and written once."""
        return (in_size * self.N * self.nb + in_size * self.n * self.n * self.d * self.n_sets
                + 2.0 * out_size * self.N * self.n_out)


def _uniform(rng, shape, lo=-1.0, hi=1.0):
    return rng.uniform(lo, hi, size=shape)


def make_batch(d: int, n: int, stride: int, n_out: int, fan_in, *, seed: int, name: str = "custom",
               block: int | None = None, input_dist: str = "normal", factor_scale: float = 1.0,
               shared_factors: bool = False, out_init: str = "zero") -> Batch:
    """Generic generator.  `fan_in` is an int (every output gets that many entries)
    or an array of per-output fan-ins.  With shared_factors, every entry of an output
    group uses the group's factor set; otherwise every entry has its own."""
    rng = np.random.Generator(np.random.PCG64(seed))
    N = n ** d
    if np.isscalar(fan_in):
        fan = np.full(n_out, int(fan_in), dtype=np.int64)
    else:
        fan = np.asarray(fan_in, dtype=np.int64)
    out_index = np.repeat(np.arange(n_out, dtype=np.int64), fan)
    nb = int(out_index.shape[0])
    block = block if block is not None else stride * max(n, 1)
    n_sets = n_out if shared_factors else nb
    factors = _uniform(rng, (n_sets * d, block)) * factor_scale
    if input_dist == "normal":
        inputs = rng.standard_normal((nb, N))
    else:
        inputs = _uniform(rng, (nb, N))
    fac_index = out_index.copy() if shared_factors else np.arange(nb, dtype=np.int64)
    if out_init == "zero":
        outs = np.zeros((n_out, N))
    else:
        outs = rng.standard_normal((n_out, N))
    return Batch(name, d, n, stride, block, factors, inputs, outs, fac_index, out_index,
                 {"seed": seed, "fan_in": fan_in if np.isscalar(fan_in) else "ragged"})


# ---- the benchmark configurations -------------------------------------------------

def config1(scale: float = 1.0, seed: int = 1001) -> Batch:
    """Plain forward FP64: d=3, n=4 (N=64), stride 4, E=1024 outputs x fan-in 8 -> 8192 entries,
    factors and inputs U[-1,1], each entry with its own factors and input, outputs zero."""
    E = max(1, int(round(1024 * scale)))
    return make_batch(3, 4, 4, E, 8, seed=seed, name="fwd_d3_n4_b8192", input_dist="uniform")


def config2(scale: float = 1.0, seed: int = 1002) -> Batch:
    """Plain forward FP64, large: d=6, n=4 (N=4096), stride 8 (each factor is the top-left 4x4
    of an 8x8 col-major block), E=4096 x fan-in 9 -> 36864 entries, factors U[-1,1], inputs N(0,1)."""
    E = max(1, int(round(4096 * scale)))
    return make_batch(6, 4, 8, E, 9, seed=seed, name="fwd_d6_n4_b36864", block=64)


CONFIG3_GROUPS = ((2, 8, 8000), (3, 6, 6000), (4, 4, 12000), (6, 3, 4000))


def config3(scale: float = 1.0, seed: int = 1003) -> list[Batch]:
    """Uneven groups (d, n, outputs) = (2,8,8000), (3,6,6000), (4,4,12000), (6,3,4000); per-output
    fan-in uniform in 1..27 (seeded), entries of one output contiguous; factors U[-1,1], inputs N(0,1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    groups = []
    for gi, (d, n, E) in enumerate(CONFIG3_GROUPS):
        E = max(1, int(round(E * scale)))
        fan = rng.integers(1, 28, size=E)
        groups.append(make_batch(d, n, n, E, fan, seed=seed * 10 + gi, name=f"group_d{d}_n{n}"))
    return groups


def config4(scale: float = 1.0, seed: int = 1004) -> Batch:
    """Reduced precision: d=4, n=8 (N=4096), 32768 entries with fan-in 8 (E=4096), factors
    U[-1,1]/8, inputs N(0,1).  Generated in FP64; the FP32 paths use a rounded copy."""
    E = max(1, int(round(4096 * scale)))
    return make_batch(4, 8, 8, E, 8, seed=seed, name="fwd_d4_n8_b32768", factor_scale=1.0 / 8)


def config5(scale: float = 1.0, seed: int = 1005) -> Batch:
    """Forward + adjoint: d=3, n=6 (N=216), 16384 entries with fan-in 8 (E=2048); the factors are
    shared by the 8 entries of an output group."""
    E = max(1, int(round(2048 * scale)))
    return make_batch(3, 6, 6, E, 8, seed=seed, name="fwdadj_d3_n6_b16384", shared_factors=True)
