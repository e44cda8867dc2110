"""Krylov solvers on a long-row matrix against the oracle (GPU).

The solvers' products with a long-row matrix (a power-law graph Laplacian)
run through the sliced SpMV with their fused epilogues (p.Ap, the
BiCGSTAB and GMRES reductions) and, in FP64, its fused-multiply-add mode;
the oracle runs the reference's loops (iterative.rs:40-162, :416-600,
:662-830) on the same system.  A = D - S with S the symmetrised absolute
power-law pattern and D its row sums plus one: symmetric and strictly
diagonally dominant, so SPD.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


@pytest.fixture(scope="module")
def ctx(S):
    c = S.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def system():
    sp = pytest.importorskip("scipy.sparse")
    ip, ix, v = O.generate("powerlaw", 6000, seed=5, param0=12.0, param1=1500.0)
    n = len(ip) - 1
    p = sp.csr_matrix((np.abs(v), ix, ip), shape=(n, n))
    s = (p + p.T) * 0.5
    s.setdiag(0.0)
    s.eliminate_zeros()
    d = np.asarray(abs(s).sum(axis=1)).ravel() + 1.0
    a = (sp.diags(d) - s).tocsr()
    a.sort_indices()
    b = O.rhs_normal(21, n)
    return a.indptr.astype(np.int64), a.indices.astype(np.int32), a.data.astype(np.float64), n, b


def test_long_rows_take_the_sliced_kernel(S, ctx, system):
    ip, ix, v, n, _ = system
    assert np.diff(ip).max() > 256
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    assert S.spmv_kernel(a) == "spmv_sliced_kernel"
    assert S.spmv_kernel(a, exact=False) == "spmv_sliced_kernel<FMA>"
    a.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_cg_jacobi_long_rows(S, ctx, system, dtype):
    ip, ix, v, n, b = system
    a = S.csr_from_arrays(ctx, ip, ix, v.astype(dtype), (n, n))
    m = S.jacobi(ctx, a)
    rtol = 1e-10 if dtype == np.float64 else 1e-5
    r = S.cg(a, b, max_iter=3000, rtol=rtol, atol=0.0, preconditioner=m)
    oa = O.op_csr_i32(ip, ix, v, (n, n), f64=dtype == np.float64)
    ro = O.cg(oa, b, max_iter=3000, rtol=rtol, atol=0.0, preconditioner=O.op_jacobi(oa))
    assert r.converged and ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= max(2, ro["iterations"] // 50)
    err = np.linalg.norm(r.x.astype(np.float64) - ro["x"]) / np.linalg.norm(ro["x"])
    assert err < (1e-8 if dtype == np.float64 else 1e-4)
    m.close()
    a.close()


def test_bicgstab_and_gmres_long_rows(S, ctx, system):
    ip, ix, v, n, b = system
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    m = S.jacobi(ctx, a)
    r = S.bicgstab(a, b, max_iter=2000, rtol=1e-10, atol=0.0, left_preconditioner=m)
    ro = O.bicgstab(oa, b, max_iter=2000, rtol=1e-10, atol=0.0, left=O.op_jacobi(oa))
    assert r.converged == ro["converged"] and r.message == ro["message"]
    assert abs(r.iterations - ro["iterations"]) <= 3
    if ro["converged"]:
        assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-7
    g = S.gmres(a, b, max_iter=2000, restart=30, rtol=1e-10, atol=0.0, preconditioner=m)
    go = O.gmres(oa, b, max_iter=2000, restart=30, rtol=1e-10, atol=0.0, preconditioner=O.op_jacobi(oa))
    assert g.converged and go["converged"]
    assert abs(g.iterations - go["iterations"]) <= max(3, go["iterations"] // 20)
    assert np.linalg.norm(g.x - go["x"]) / np.linalg.norm(go["x"]) < 1e-8
    m.close()
    a.close()
