"""ZeroOperator, SumOperator and ProductOperator (linalg/interface.rs:177-402)
on the device: results, adjoints, errors, and use inside a solver."""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _csr(S, ctx, kind="aniso_q1", dims=(40, 30, 1)):
    ip, ix, v = S.generate(kind, *dims, seed=1, param0=20.0, param1=0.5)
    n = len(ip) - 1
    return ip, ix, v, S.csr_from_arrays(ctx, ip, ix, v, (n, n))


def test_zero_operator(S, ctx):
    z = S.zero_operator(ctx, 3, 5)
    assert z.shape == (3, 5) and z.has_adjoint
    assert np.array_equal(z.matvec(np.full(5, np.inf)), np.zeros(3))  # interface.rs:207
    assert np.array_equal(z.rmatvec(np.ones(3)), np.zeros(5))
    with pytest.raises(S.SparseError) as e:
        z.matvec(np.ones(3))
    assert e.value.variant == "DimensionMismatch"
    z.close()


def test_sum_and_product_bit_exact(S, ctx):
    ip, ix, v, a = _csr(S, ctx)
    n = a.shape[0]
    rng = np.random.default_rng(3)
    d = rng.uniform(0.5, 2.0, n)
    x = rng.standard_normal(n)
    dg = S.diagonal(ctx, d)
    s = S.sum_operator(a, dg)
    p = S.product_operator(a, dg)
    # (A + D) x = A x + D x, each rounded like the reference (interface.rs:325-329)
    assert np.array_equal(s.matvec(x).view(np.uint8), (O.spmv_i32(ip, ix, v, x) + x * d).view(np.uint8))
    # (A D) x = A (D x) (interface.rs:377-380)
    assert np.array_equal(p.matvec(x).view(np.uint8), O.spmv_i32(ip, ix, v, x * d).view(np.uint8))
    # adjoints: (A + D)^T x = A^T x + D x, (A D)^T x = D (A^T x)
    at = a.rmatvec(x)
    assert np.array_equal(s.rmatvec(x).view(np.uint8), (at + x * d).view(np.uint8))
    assert np.array_equal(p.rmatvec(x).view(np.uint8), (at * d).view(np.uint8))
    for op in (s, p, dg, a):
        op.close()


def test_composite_errors(S, ctx):
    a3 = S.identity(ctx, 3)
    z23 = S.zero_operator(ctx, 2, 3)
    with pytest.raises(S.SparseError) as e:
        S.sum_operator(a3, z23)
    assert e.value.variant == "ShapeMismatch"
    assert str(e.value) == "Shape mismatch: expected (3, 3), found (2, 3)"
    z32 = S.zero_operator(ctx, 3, 2)
    with pytest.raises(S.SparseError) as e:
        S.product_operator(z32, S.zero_operator(ctx, 3, 3))
    assert e.value.variant == "DimensionMismatch"
    assert str(e.value) == "Dimension mismatch: expected 2, found 3"
    # a host operator has no adjoint (the trait's default), so neither does the sum
    h = S.host_operator(ctx, 3, lambda x: 2.0 * x)
    s = S.sum_operator(a3, h)
    assert not s.has_adjoint
    assert np.allclose(s.matvec(np.array([1.0, 2.0, 3.0])), [3.0, 6.0, 9.0])
    with pytest.raises(S.SparseError) as e:
        s.rmatvec(np.ones(3))
    assert e.value.variant == "OperationNotSupported"
    assert str(e.value) == "Operation not supported: adjoint not supported for one or both operators"
    for op in (s, h, z32, z23, a3):
        op.close()


def test_cg_on_a_shifted_operator(S, ctx):
    # cg on A + 0.5 I given as a SumOperator (captured into the solver graph)
    ip, ix, v, a = _csr(S, ctx)
    n = a.shape[0]
    sh = S.scaled_identity(ctx, n, 0.5)
    op = S.sum_operator(a, sh)
    b = S.rhs_normal(2, n)
    r = S.cg(op, b, max_iter=5000, rtol=1e-10, atol=0.0)
    assert r.converged
    res = op.matvec(r.x) - b
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(b)
    for o in (op, sh, a):
        o.close()
