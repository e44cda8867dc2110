"""IC(0) on the device vs the oracle's restatement of ic.rs (bit-exact apply)."""
import numpy as np
import pytest

from oracle import oracle_ffi as O
from tests import reference_cases as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def test_ic0_reference_cases(S, ctx):
    c = R.IC0_SPD
    a = S.csr_matrix_from_raw(ctx, c["data"], c["indptr"], c["indices"], (3, 3))
    m = S.ic0(ctx, a)
    y = m.matvec(c["b"])
    assert np.all(np.isfinite(y))
    oa = O.op_csr(c["indptr"], c["indices"], np.asarray(c["data"]), (3, 3))
    assert np.array_equal(y, O.op_ic0(oa).matvec(c["b"]))
    c = R.IC0_NOT_SPD
    a = S.csr_matrix_from_raw(ctx, c["data"], c["indptr"], c["indices"], (2, 2))
    with pytest.raises(S.SparseError) as e:
        S.ic0(ctx, a)
    assert str(e.value) == "Value error: Matrix is not positive definite or factorization broke down"


def test_ic0_missing_diagonal(S, ctx):
    a = S.csr_matrix(ctx, [4.0, 1.0, 1.0], [0, 1, 1], [0, 0, 2], (3, 3))
    with pytest.raises(S.SparseError) as e:
        S.ic0(ctx, a)
    assert str(e.value) == "Value error: Missing diagonal element at position 1"


def test_ic0_reference_breakdown_on_variable_coefficients(S, ctx):
    # The reference factorisation subtracts a_ij^2 / L_jj (ic.rs:94) instead of
    # a_ij^2 / L_jj^2 and breaks down on variable-coefficient diffusion; the
    # device reports the same error, the textbook variant succeeds.
    ip, ix, v = S.generate("varcoef3d", 12, 10, 9, seed=2, param0=1.5)
    n = len(ip) - 1
    oa = O.op_csr(ip.astype(np.uint64), ix.astype(np.uint64), v, (n, n))
    with pytest.raises(ValueError) as eo:
        O.op_ic0(oa)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    with pytest.raises(S.SparseError) as ed:
        S.ic0(ctx, a)
    assert str(ed.value) == str(eo.value)
    m = S.ic0(ctx, a, textbook=True)
    assert np.all(np.isfinite(m.matvec(S.rhs_normal(1, n))))


@pytest.mark.parametrize("kind,dims,p0,p1,dtype", [
    ("poisson2d", (40, 30, 1), 0.0, 0.0, np.float64),
    ("laplace3d", (12, 10, 9), 0.0, 0.0, np.float64),
    ("aniso_q1", (33, 29, 1), 50.0, 0.4, np.float64),
    ("poisson2d", (40, 30, 1), 0.0, 0.0, np.float32),
])
def test_ic0_apply_bit_exact(S, ctx, kind, dims, p0, p1, dtype):
    ip, ix, v = S.generate(kind, *dims, seed=2, param0=p0, param1=p1)
    n = len(ip) - 1
    vals = v.astype(dtype)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    m = S.ic0(ctx, a)
    oa = O.op_csr(ip.astype(np.uint64), ix.astype(np.uint64), vals, (n, n))
    om = O.op_ic0(oa)
    x = S.rhs_normal(5, n).astype(dtype)
    assert np.array_equal(m.matvec(x).view(np.uint8), om.matvec(x).view(np.uint8))


def test_ic0_unsorted_and_duplicate_entries_bit_exact(S, ctx):
    # rows stored out of order with a duplicated diagonal exercise the
    # reference's post-diagonal update loop (ic.rs:107-128)
    rng = np.random.default_rng(8)
    n = 50
    rows, cols, vals = [], [], []
    for i in range(n):
        ent = [(i, 8.0 + rng.uniform())]
        for j in rng.choice(i, min(i, 3), replace=False) if i else []:
            ent.append((int(j), -rng.uniform(0.1, 0.5)))
        if i % 7 == 3:
            ent.append((i, 0.5))  # duplicated diagonal
        rng.shuffle(ent)
        for j, val in ent:
            rows.append(i); cols.append(j); vals.append(val)
    ip = np.zeros(n + 1, dtype=np.uint64)
    for r in rows:
        ip[r + 1] += 1
    ip = np.cumsum(ip).astype(np.uint64)
    a = S.csr_array(ctx, vals, cols, ip, (n, n))
    assert not a.has_sorted_indices
    m = S.ic0(ctx, a)
    om = O.op_ic0(O.op_csr(ip, np.asarray(cols, dtype=np.uint64), np.asarray(vals), (n, n)))
    x = S.rhs_normal(1, n)
    assert np.array_equal(m.matvec(x), om.matvec(x))


def test_textbook_ic0_is_a_better_factor(S, ctx):
    ip, ix, v = S.generate("poisson2d", 32, 32)
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    b = S.rhs_normal(3, n)
    r_ref = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.ic0(ctx, a))
    r_txt = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.ic0(ctx, a, textbook=True))
    r_jac = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.jacobi(ctx, a))
    assert r_ref.converged and r_txt.converged and r_jac.converged
    assert r_txt.iterations < r_jac.iterations


def test_cg_with_ic0_matches_oracle(S, ctx):
    ip, ix, v = S.generate("aniso_q1", 30, 25, seed=4, param0=20.0, param1=0.3)
    n = len(ip) - 1
    b = S.rhs_normal(4, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.ic0(ctx, a))
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    ro = O.cg(oa, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=O.op_ic0(oa))
    assert r.converged == ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= 2
    if r.converged:
        assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-8
