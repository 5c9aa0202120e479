"""The hand-written adjoint kernel: grad_input against the reference applied with
transposed factors (golden fixture and oracle), grad_A against an explicit
mode-unfolding formula, and both against central finite differences through the
torch.autograd wrapper."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def factor(b, row):
    A = b.factors[row]
    return np.array([[A[r + c * b.stride] for c in range(b.n)] for r in range(b.n)])


def transposed_batch(b, grad_out):
    """Batch whose forward is the adjoint's grad_input: factors A^T (stride n), inputs g[out(k)]."""
    from kronmult_gb300.workloads import Batch

    fac_t = np.stack([factor(b, r).T.reshape(-1, order="F") for r in range(b.factors.shape[0])])
    return Batch(b.name + "_T", b.d, b.n, b.n, b.n * b.n, fac_t, grad_out[b.out_index], np.zeros((b.nb, b.N)),
                 b.fac_index, np.arange(b.nb, dtype=np.int64))


def apply_mode(T, A, axis):
    return np.moveaxis(np.tensordot(A, T, axes=([1], [axis])), 0, axis)


def grad_factors_numpy(b, grad_out):
    """dL/dA for L = sum_e <g_e, out_e>, by the mode-unfolding formula, per factor row."""
    n, d = b.n, b.d
    G = np.zeros((b.factors.shape[0], n, n))
    for k in range(b.nb):
        A = [factor(b, b.fac_index[k] * d + i) for i in range(d)]
        X = b.inputs[k].reshape((n,) * d)
        Gt = grad_out[b.out_index[k]].reshape((n,) * d)
        for i in range(d):
            U = X
            for m in range(d):
                if m != i:
                    U = apply_mode(U, A[m], m)
            axes = [a for a in range(d) if a != i]
            G[b.fac_index[k] * d + i] += np.tensordot(np.moveaxis(Gt, i, 0), np.moveaxis(U, i, 0),
                                                      axes=(list(range(1, d)), list(range(1, d))))
    return G


def run_adjoint(b, grad_out, cuda, dtype=torch.float64, want_gin=True, want_gA=True, tuning=None):
    from kronmult_gb300 import DeviceBatch, adjoint

    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype)
    g = torch.from_numpy(grad_out).to(cuda, dtype)
    gin = torch.zeros_like(db.inputs) if want_gin else None
    gfa = torch.zeros_like(db.factors) if want_gA else None
    adjoint(db, g, gin, gfa, tuning=tuning)
    torch.cuda.synchronize()
    gA = None
    if gfa is not None:
        gfa = gfa.cpu().numpy()
        gA = np.stack([np.array([[row[r + c * b.stride] for c in range(b.n)] for r in range(b.n)]) for row in gfa])
    return (gin.cpu().numpy() if gin is not None else None), gA


def test_grad_input_golden_c5(cuda):
    b, z = load_golden("c5_small")
    gin, _ = run_adjoint(b, z["grad_out"], cuda, want_gA=False)
    assert O.rel_l2(gin, z["expected_grad_input_f64"]) <= 1e-13


@pytest.mark.parametrize("d,n", [(1, 2), (2, 8), (3, 6), (4, 4), (6, 3), (3, 5), (2, 7), (5, 2), (6, 4), (2, 9),
                                 (2, 12), (3, 3)])
def test_adjoint_shapes_f64(cuda, d, n):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 1, 3, 4, seed=100 + 10 * d + n, shared_factors=True)
    g = np.random.Generator(np.random.PCG64(5)).standard_normal((b.n_out, b.N))
    gin, gA = run_adjoint(b, g, cuda)
    assert O.rel_l2(gin, O.forward(transposed_batch(b, g))) <= 1e-13
    assert O.rel_l2(gA, grad_factors_numpy(b, g)) <= 1e-13


def test_adjoint_config2_shape_recompute_path(cuda):
    """d=6, n=4 in FP64 does not fit all partial products in shared memory: the
    kernel rebuilds each one from x."""
    from kronmult_gb300 import workloads as W

    b = W.config2(scale=2 / 4096)
    g = np.random.Generator(np.random.PCG64(6)).standard_normal((b.n_out, b.N))
    gin, gA = run_adjoint(b, g, cuda)
    assert O.rel_l2(gin, O.forward(transposed_batch(b, g))) <= 1e-13
    assert O.rel_l2(gA, grad_factors_numpy(b, g)) <= 1e-12


def test_adjoint_config5_f32(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config5(scale=8 / 2048)
    g = np.random.Generator(np.random.PCG64(7)).standard_normal((b.n_out, b.N))
    gin, gA = run_adjoint(b, g, cuda, dtype=torch.float32)
    assert O.rel_l2(gin, O.forward(transposed_batch(b, g))) <= 1e-5
    assert O.rel_l2(gA, grad_factors_numpy(b, g)) <= 1e-5


@pytest.mark.parametrize("team_size", [8, 16, 32, 64, 128])
def test_adjoint_team_sizes(cuda, team_size):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(3, 6, 6, 5, 3, seed=77, shared_factors=True)
    g = np.random.Generator(np.random.PCG64(8)).standard_normal((b.n_out, b.N))
    gin, gA = run_adjoint(b, g, cuda, tuning={"team_size": team_size, "entries_per_team": 2})
    assert O.rel_l2(gin, O.forward(transposed_batch(b, g))) <= 1e-13
    assert O.rel_l2(gA, grad_factors_numpy(b, g)) <= 1e-13


def test_autograd_central_differences(cuda):
    """backward of the autograd wrapper against central finite differences
    (h = 1e-6, FP64) of the CPU oracle's forward, along random directions."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.autograd import KronSpec, kronmult
    from kronmult_gb300.workloads import Batch

    b = W.config5(scale=4 / 2048)
    rng = np.random.Generator(np.random.PCG64(9))
    g = rng.standard_normal((b.n_out, b.N))
    fac = torch.from_numpy(b.factors).to(cuda).requires_grad_(True)
    x = torch.from_numpy(b.inputs).to(cuda).requires_grad_(True)
    spec = KronSpec(b.d, b.n, b.stride, b.n_out, torch.from_numpy(b.fac_index).to(cuda),
                    torch.from_numpy(b.out_index).to(cuda))
    out = kronmult(fac, x, spec)
    assert O.rel_l2(out.detach().cpu().numpy(), O.forward(b)) <= 1e-13
    (out * torch.from_numpy(g).to(cuda)).sum().backward()

    def loss(factors, inputs):
        bb = Batch(b.name, b.d, b.n, b.stride, b.block, factors, inputs, np.zeros_like(b.out_init), b.fac_index,
                   b.out_index)
        return float((O.forward(bb) * g).sum())

    h = 1e-6
    for _ in range(3):
        vx = rng.standard_normal(b.inputs.shape)
        fd = (loss(b.factors, b.inputs + h * vx) - loss(b.factors, b.inputs - h * vx)) / (2 * h)
        an = float((x.grad.cpu().numpy() * vx).sum())
        assert abs(fd - an) <= 1e-7 * max(1.0, abs(an))
        # perturb one factor row at a time: L is linear in each factor separately
        row = int(rng.integers(0, b.factors.shape[0]))
        vA = np.zeros_like(b.factors)
        vA[row] = rng.standard_normal(b.factors.shape[1])
        fd = (loss(b.factors + h * vA, b.inputs) - loss(b.factors - h * vA, b.inputs)) / (2 * h)
        mask = np.zeros(b.factors.shape[1], dtype=bool)
        for c in range(b.n):
            mask[c * b.stride:c * b.stride + b.n] = True  # only the n x n entries are used
        an = float((fac.grad.cpu().numpy()[row][mask] * vA[row][mask]).sum())
        assert abs(fd - an) <= 1e-7 * max(1.0, abs(an))


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-13), (torch.float32, 1e-5)])
def test_adjoint_balanced_ranges_large_batch(cuda, dtype, tol):
    """More entries than team slots (8192 entries, d=3, n=6): by default every slot of
    one wave takes an equal share of the entries; fixed runs of 4 entries per team give
    the same gradients up to summation order, and grad_input matches the oracle."""
    from kronmult_gb300 import workloads as W

    b = W.config5(scale=1024 / 2048)
    g = np.random.Generator(np.random.PCG64(10)).standard_normal((b.n_out, b.N))
    gin, gA = run_adjoint(b, g, cuda, dtype=dtype)
    gin_r, gA_r = run_adjoint(b, g, cuda, dtype=dtype, tuning={"entries_per_team": 4})
    assert O.rel_l2(gin, gin_r) <= tol
    assert O.rel_l2(gA, gA_r) <= tol
    assert O.rel_l2(gin, O.forward(transposed_batch(b, g))) <= tol
