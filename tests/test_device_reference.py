"""The reference crate's own tests, replayed through the device library's C ABI."""
import numpy as np
import pytest

from tests import reference_cases as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def test_csr_create_dense_dot_transpose(S, ctx):
    c = R.CSR_BASIC
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], c["shape"])
    assert a.shape == (3, 3) and a.nnz == 5
    assert np.array_equal(a.to_dense(), c["dense"])
    assert np.allclose(a.matvec(c["dot_x"]), c["dot_y"], atol=1e-10)
    t = a.transpose()
    assert t.shape == (3, 3) and t.nnz == 5
    assert np.array_equal(t.to_dense(), c["dense_t"])


def test_csr_array_new_from_triplets_dot_vector(S, ctx):
    c = R.CSR_ARRAY
    a = S.csr_array(ctx, c["data"], c["indices"], c["indptr"], c["shape"])
    b = S.csr_array_from_triplets(ctx, c["rows"], c["cols"], c["data"], c["shape"])
    for m in (a, b):
        assert m.shape == (3, 3) and m.nnz == 5
        for (i, j), v in c["gets"]:
            assert m.get(i, j) == v
        assert np.allclose(m.matvec(c["dot_x"]), c["dot_y"])


def test_cg_identity_and_diagonal(S, ctx):
    r = S.cg(S.identity(ctx, 3), R.IDENTITY_B)
    assert r.converged and np.allclose(r.x, R.IDENTITY_B, atol=1e-10)
    r = S.cg(S.diagonal(ctx, R.DIAG["diag"]), R.DIAG["b"])
    assert r.converged and np.allclose(r.x, R.DIAG["x"], atol=1e-10)


def test_bicgstab_identity_and_diagonal(S, ctx):
    r = S.bicgstab(S.identity(ctx, 3), R.IDENTITY_B)
    assert r.converged and np.allclose(r.x, R.IDENTITY_B, atol=1e-10)
    r = S.bicgstab(S.diagonal(ctx, R.DIAG["diag"]), R.DIAG["b"])
    assert r.converged and np.allclose(r.x, R.DIAG["x"], atol=1e-10)


def test_cg_sparse_3x3(S, ctx):
    c = R.SPD3
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], (3, 3))
    r = S.cg(a, c["b"])
    assert r.converged
    assert np.all(np.abs(a.matvec(r.x) - c["b"]) < c["tol"])


def test_bicgstab_non_symmetric(S, ctx):
    c = R.NONSYM3
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], (3, 3))
    r = S.bicgstab(a, c["b"])
    assert r.converged
    assert np.all(np.abs(a.matvec(r.x) - c["b"]) < c["tol"])


def test_cg_2x2(S, ctx):
    c = R.CG_2X2
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], (2, 2))
    r = S.cg(a, c["b"])
    assert r.converged and np.allclose(r.x, c["x"], atol=c["tol"])


def test_cg_with_jacobi(S, ctx):
    c = R.CG_JACOBI
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], (3, 3))
    r = S.cg(a, c["b"], preconditioner=S.jacobi(ctx, a))
    assert r.converged and r.iterations < c["max_iterations"]
    assert np.allclose(a.matvec(r.x), c["b"], atol=c["tol"])


def test_jacobi_apply(S, ctx):
    c = R.JACOBI_APPLY
    m = S.jacobi_from_diagonal(ctx, c["diag"])
    assert np.allclose(m.matvec(c["x"]), c["y"], atol=1e-10)
    a = S.csr_matrix(ctx, c["diag"], [0, 1, 2], [0, 1, 2], (3, 3))
    assert np.allclose(S.jacobi(ctx, a).matvec(c["x"]), c["y"], atol=1e-10)


def test_bicgstab_duplicate_entry_with_jacobi(S, ctx):
    c = R.BICGSTAB_DUP
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], c["shape"])
    m = S.jacobi(ctx, a)
    assert np.isclose(m.matvec([0, 0, 0, 1.0])[3], 1.0 / 15.0)
    assert np.isclose(a.matvec([0, 0, 0, 1.0])[3], 16.0)
    r = S.bicgstab(a, c["b"], max_iter=c["max_iter"], rtol=c["rtol"], atol=c["atol"],
                   left_preconditioner=m)
    assert r.converged and r.iterations < c["max_iterations"]
    assert np.linalg.norm(np.asarray(c["b"]) - a.matvec(r.x)) < c["resid"]


def test_bicgstab_convection_diffusion(S, ctx):
    c = R.convection_diffusion()
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], c["shape"])
    r = S.bicgstab(a, c["b"], max_iter=c["max_iter"], rtol=c["rtol"], atol=c["atol"])
    assert r.converged
    assert np.linalg.norm(np.asarray(c["b"]) - a.matvec(r.x)) < c["resid"]


def test_bicgstab_breakdown(S, ctx):
    c = R.SINGULAR
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], c["shape"])
    r = S.bicgstab(a, c["b"])
    assert not r.converged and "breakdown" in r.message


def test_gmres_small_systems(S, ctx):
    c = R.NONSYM3
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], (3, 3))
    r = S.gmres(a, c["b"])
    assert r.converged and np.all(np.abs(a.matvec(r.x) - c["b"]) < 1e-9)
    c = R.convection_diffusion()
    a = S.csr_matrix(ctx, c["data"], c["rows"], c["cols"], c["shape"])
    r = S.gmres(a, c["b"], restart=4)
    assert r.converged and np.linalg.norm(np.asarray(c["b"]) - a.matvec(r.x)) < 1e-6


def test_construction_errors(S, ctx):
    with pytest.raises(S.SparseError) as e:
        S.csr_matrix(ctx, [1.0, 2.0], [0, 3], [0, 0], (3, 3))
    assert e.value.variant == "ValueError" and str(e.value) == "Value error: Row index out of bounds"
    with pytest.raises(S.SparseError) as e:
        S.csr_matrix(ctx, [1.0, 2.0], [0, 1], [0, 5], (3, 3))
    assert str(e.value) == "Value error: Column index out of bounds"
    with pytest.raises(S.SparseError) as e:
        S.csr_array_from_triplets(ctx, [0, 4, 5], [0, 0, 9], [1.0, 2.0, 3.0], (3, 3))
    assert e.value.variant == "IndexOutOfBounds"
    assert str(e.value) == "Index (4, 0) out of bounds for array with shape (3, 3)"
    with pytest.raises(S.SparseError) as e:
        S.csr_matrix_from_raw(ctx, [1.0, 2.0], [0, 2, 1], [0, 1], (2, 2))
    assert str(e.value) == "Value error: Row pointer array must be monotonically increasing"
    with pytest.raises(S.SparseError) as e:
        S.csr_array(ctx, [1.0], [0], [1, 1], (1, 1))
    assert str(e.value) == "Inconsistent data: first element of indptr must be 0"
    with pytest.raises(S.SparseError) as e:
        S.jacobi(ctx, S.csr_matrix(ctx, [1.0, 1.0], [0, 1], [1, 0], (2, 2)))
    assert str(e.value) == "Value error: Zero diagonal element at position 0"


def test_solver_shape_errors(S, ctx):
    a = S.csr_matrix(ctx, [1.0, 2.0], [0, 1], [0, 2], (2, 3))
    with pytest.raises(S.SparseError) as e:
        S.cg(a, [1.0, 2.0])
    assert str(e.value) == "Value error: Matrix must be square for CG solver"
    b = S.csr_matrix(ctx, [1.0, 2.0], [0, 1], [0, 1], (2, 2))
    with pytest.raises(S.SparseError) as e:
        S.bicgstab(b, [1.0, 2.0, 3.0])
    assert e.value.variant == "DimensionMismatch" and e.value.payload[:2] == (2, 3)


def test_cg_zero_rhs_reports_not_positive_definite(S, ctx):
    # iterative.rs:96-110: cg checks no initial convergence, so b = 0 gives pAp = 0
    a = S.csr_matrix(ctx, [2.0, 2.0], [0, 1], [0, 1], (2, 2))
    r = S.cg(a, [0.0, 0.0])
    assert not r.converged and r.iterations == 0
    assert r.message == "Matrix not positive definite (p^T*A*p <= 0)"


def test_max_iter_zero(S, ctx):
    a = S.csr_matrix(ctx, [2.0, 2.0], [0, 1], [0, 1], (2, 2))
    r = S.cg(a, [1.0, 1.0], max_iter=0)
    assert not r.converged and r.iterations == 0 and r.message == "Maximum iterations reached"
    r = S.bicgstab(a, [1.0, 1.0], max_iter=0)
    assert r.message == "Maximum iterations reached"
    r = S.bicgstab(a, [0.0, 0.0])
    assert r.converged and r.message == "Converged with initial guess"
