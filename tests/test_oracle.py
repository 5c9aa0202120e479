"""The CPU oracle pinned to the reference's own outputs (golden fixtures) and to
the explicit-Kronecker definition.  No GPU needed."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as O


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden_f64(name):
    b, z = load_golden(name)
    got = O.forward(b, impl="port", nthreads=1)
    # same operation order as kronmult_omp; only FMA contraction may differ by platform
    assert O.rel_l2(got, z["expected_f64"]) <= 1e-15


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden_f32(name):
    b, z = load_golden(name)
    got = O.forward(b, dtype=np.float32, impl="port", nthreads=1)
    assert O.rel_l2(got, z["expected_f32"]) <= 1e-6


@pytest.mark.parametrize("name", [n for n in golden_names() if n not in ("n2_d10",)])
def test_naive_definition(name):
    """The sweep equals the explicit Kronecker matrix-vector product."""
    b, z = load_golden(name)
    if b.N > 1024:
        pytest.skip("explicit Kronecker matrix too large")
    naive = O.forward(b, impl="naive")
    assert O.rel_l2(naive, z["expected_f64"]) <= 1e-14


def test_golden_index_convention():
    """kron(A_0,...,A_{d-1}) has A_0 as the most significant index
    (tests/utils/kronmult_naive.h:60-61): check with numpy's kron."""
    b, z = load_golden("n3_d3_stride5")
    k = 0
    mats = []
    for i in range(b.d):
        A = b.factors[b.fac_index[k] * b.d + i]
        mats.append(np.array([[A[r + c * b.stride] for c in range(b.n)] for r in range(b.n)]))
    K = mats[0]
    for M in mats[1:]:
        K = np.kron(K, M)
    y = K @ b.inputs[k]
    single = type(b)(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs[:1], np.zeros((1, b.N)),
                     b.fac_index[:1], np.zeros(1, dtype=np.int64))
    assert O.rel_l2(O.forward(single), y[None, :]) <= 1e-15


def test_reference_naive_d1_agrees():
    """The reference's own naive check, usable for d == 1 only (for d >= 2 its
    kronmult_naive allocates size_kron*n values for a (size_kron*n)^2 matrix)."""
    if not O.available("reference"):
        pytest.skip("reference not built here")
    b, z = load_golden("toy")
    assert O.rel_l2(O.forward(b, impl="reference_naive"), z["expected_f64"]) <= 1e-15


def test_empty_batch_is_noop():
    b, z = load_golden("empty_batch")
    assert O.forward(b).shape == (0, b.N)


@pytest.mark.parametrize("d,n", [(0, 3), (0, 1), (1, 1), (3, 1), (1, 2), (2, 9), (2, 12), (3, 10)])
def test_edge_shapes_against_definition(d, n):
    """d = 0 (the empty product, out += in), n = 1 and n > 8: the sweep against the
    explicit Kronecker product, and against the reference build where it is present."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 2, 5, 3, seed=930 + 10 * d + n, out_init="normal")
    got = O.forward(b)
    assert O.rel_l2(got, O.forward(b, impl="naive")) <= 1e-14
    if d == 0:
        want = b.out_init.copy()
        np.add.at(want, b.out_index, b.inputs)
        assert O.rel_l2(got, want) <= 1e-15  # only the order of the additions differs
    if O.available("reference"):
        assert O.rel_l2(got, O.forward(b, impl="reference")) <= 1e-15
