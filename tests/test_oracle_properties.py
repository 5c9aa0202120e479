"""Size-independent properties of the batched Kronecker product, checked on the CPU
oracle (the checker the CUDA paths are compared with): linearity in the inputs, the
adjoint identity <K x, g> = <x, K^T g> with K^T applied as the same batched product of
transposed factors, additivity over aliased outputs, and the Kronecker mixed-product
rule kron(A, B) kron(C, D) = kron(AC, BD) through two chained products."""
import numpy as np
import pytest

from oracle import oracle as O

SHAPES = [(1, 5), (2, 3), (3, 4), (2, 7), (4, 2), (3, 6)]


def _batch(d, n, seed, n_out=3, fan=4, stride=None):
    from kronmult_gb300 import workloads as W

    return W.make_batch(d, n, stride or n + 1, n_out, fan, seed=seed)


def _with(b, **kw):
    from kronmult_gb300.workloads import Batch

    f = dict(name=b.name, d=b.d, n=b.n, stride=b.stride, block=b.block, factors=b.factors, inputs=b.inputs,
             out_init=b.out_init, fac_index=b.fac_index, out_index=b.out_index)
    f.update(kw)
    return Batch(**f)


def _factor(b, row):
    A = b.factors[row]
    return np.array([[A[r + c * b.stride] for c in range(b.n)] for r in range(b.n)])


def _transposed(b, g):
    """Batch whose forward is grad_input: factors A^T (stride n), inputs g[out(k)], one output per entry."""
    fac_t = np.stack([_factor(b, r).T.reshape(-1, order="F") for r in range(b.factors.shape[0])])
    return _with(b, stride=b.n, block=b.n * b.n, factors=fac_t, inputs=g[b.out_index],
                 out_init=np.zeros((b.nb, b.N)), out_index=np.arange(b.nb, dtype=np.int64))


@pytest.mark.parametrize("d,n", SHAPES)
def test_linearity_in_the_inputs(d, n):
    b = _batch(d, n, seed=300 + 10 * d + n)
    rng = np.random.Generator(np.random.PCG64(d * 31 + n))
    y = rng.standard_normal(b.inputs.shape)
    al, be = 0.75, -1.5
    zero = np.zeros_like(b.out_init)
    fx = O.forward(_with(b, out_init=zero))
    fy = O.forward(_with(b, inputs=y, out_init=zero))
    fxy = O.forward(_with(b, inputs=al * b.inputs + be * y, out_init=zero))
    assert O.rel_l2(fxy, al * fx + be * fy) <= 1e-13


@pytest.mark.parametrize("d,n", SHAPES)
def test_adjoint_identity(d, n):
    b = _batch(d, n, seed=400 + 10 * d + n)
    g = np.random.Generator(np.random.PCG64(d * 17 + n)).standard_normal((b.n_out, b.N))
    kx = O.forward(_with(b, out_init=np.zeros_like(b.out_init)))
    ktg = O.forward(_transposed(b, g))  # row k: K_k^T g_{out(k)}
    lhs = float(np.sum(kx * g))
    rhs = float(np.sum(b.inputs * ktg))
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))


@pytest.mark.parametrize("d,n", SHAPES)
def test_aliased_outputs_add_up(d, n):
    """Entries aliased onto one output give the sum of the same entries written to
    distinct outputs (the atomic epilogue's contract)."""
    b = _batch(d, n, seed=500 + 10 * d + n, n_out=1, fan=6)
    sep = O.forward(_with(b, out_init=np.zeros((b.nb, b.N)), out_index=np.arange(b.nb, dtype=np.int64)))
    ali = O.forward(_with(b, out_init=np.zeros((1, b.N))))
    assert O.rel_l2(ali[0], sep.sum(axis=0)) <= 1e-13


@pytest.mark.parametrize("n", [2, 3, 4])
def test_mixed_product_rule(n):
    """Applying kron(C, D) then kron(A, B) equals applying kron(AC, BD): two chained
    d = 2 products against one product of the multiplied factors."""
    rng = np.random.Generator(np.random.PCG64(600 + n))
    A, B, C, D = (rng.uniform(-1, 1, (n, n)) for _ in range(4))
    x = rng.standard_normal(n * n)

    def one(F0, F1, v):
        from kronmult_gb300.workloads import Batch

        fac = np.stack([F0.reshape(-1, order="F"), F1.reshape(-1, order="F")])
        bb = Batch("mp", 2, n, n, n * n, fac, v[None, :], np.zeros((1, n * n)), np.zeros(1, dtype=np.int64),
                   np.zeros(1, dtype=np.int64))
        return O.forward(bb)[0]

    chained = one(A, B, one(C, D, x))
    direct = one(A @ C, B @ D, x)
    assert O.rel_l2(chained, direct) <= 1e-13
    assert O.rel_l2(direct, np.kron(A @ C, B @ D) @ x) <= 1e-13
