"""The CPU oracle replays the reference crate's own tests (pins the oracle).

Every assertion mirrors the one in the cited Rust test; where the reference
only asserts a property (convergence, a residual bound), the same property is
asserted here.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_ffi as O
from tests import reference_cases as R


def csr_new(rows, cols, data, shape, f64=True):
    dt = np.float64 if f64 else np.float32
    rows = np.asarray(rows, dtype=np.uint64)
    cols = np.asarray(cols, dtype=np.uint64)
    data = np.asarray(data, dtype=dt)
    nnz = len(data)
    indptr = np.empty(shape[0] + 1, dtype=np.uint64)
    indices = np.empty(nnz, dtype=np.uint64)
    out = np.empty(nnz, dtype=dt)
    e = O.Err()
    f = O.lib().or_csr_matrix_new_f64 if f64 else O.lib().or_csr_matrix_new_f32
    rc = f(O.p(data), O.p(rows), O.p(cols), nnz, shape[0], shape[1], O.p(indptr), O.p(indices),
           O.p(out), C.byref(e))
    return rc, e.msg.decode(), indptr, indices, out


def dense(indptr, indices, data, shape):
    d = np.zeros(shape)
    for r in range(shape[0]):
        for k in range(int(indptr[r]), int(indptr[r + 1])):
            d[r, int(indices[k])] = data[k]
    return d


def test_csr_create_dense_dot_transpose():
    c = R.CSR_BASIC
    rc, _, ip, ix, d = csr_new(c["rows"], c["cols"], c["data"], c["shape"])
    assert rc == 0 and len(d) == 5
    assert np.array_equal(dense(ip, ix, d, c["shape"]), c["dense"])
    y = np.empty(3)
    x = np.asarray(c["dot_x"])
    O.lib().or_spmv_f64(O.p(ip), O.p(ix), O.p(d), 3, O.p(x), O.p(y))
    assert np.allclose(y, c["dot_y"], atol=1e-10)
    tp = np.empty(4, dtype=np.uint64)
    ti = np.empty(5, dtype=np.uint64)
    td = np.empty(5)
    O.lib().or_csr_transpose_f64(O.p(ip), O.p(ix), O.p(d), 3, 3, O.p(tp), O.p(ti), O.p(td))
    assert np.array_equal(dense(tp, ti, td, (3, 3)), c["dense_t"])


def test_csr_array_new_from_triplets_dot_vector():
    c = R.CSR_ARRAY
    ip = np.asarray(c["indptr"], dtype=np.uint64)
    ix = np.asarray(c["indices"], dtype=np.uint64)
    s, e = C.c_int(), O.Err()
    assert O.lib().or_csr_array_new_check(O.p(ip), 4, O.p(ix), 5, 5, 3, 3, C.byref(s), C.byref(e)) == 0
    assert s.value == 1
    d = np.asarray(c["data"])
    for (i, j), v in c["gets"]:
        assert O.lib().or_csr_get_f64(O.p(ip), O.p(ix), O.p(d), 3, 3, i, j) == v
    # from_triplets gives the same arrays
    rows = np.asarray(c["rows"], dtype=np.uint64)
    cols = np.asarray(c["cols"], dtype=np.uint64)
    oip = np.empty(4, dtype=np.uint64)
    oix = np.empty(5, dtype=np.uint64)
    od = np.empty(5)
    rc = O.lib().or_csr_array_from_triplets_f64(O.p(rows), O.p(cols), O.p(d), 5, 3, 3, 0, O.p(oip),
                                                O.p(oix), O.p(od), C.byref(s), C.byref(e))
    assert rc == 0
    assert np.array_equal(oip, ip) and np.array_equal(oix, ix) and np.array_equal(od, d)
    y = np.empty(3)
    x = np.asarray(c["dot_x"])
    O.lib().or_spmv_f64(O.p(ip), O.p(ix), O.p(d), 3, O.p(x), O.p(y))
    assert np.allclose(y, c["dot_y"])


def op_from_triplets(rows, cols, data, shape):
    rc, msg, ip, ix, d = csr_new(rows, cols, data, shape)
    assert rc == 0, msg
    return O.op_csr(ip, ix, d, shape)


def test_cg_identity_and_diagonal():
    r = O.cg(O.op_identity(3), R.IDENTITY_B)
    assert r["converged"] and np.allclose(r["x"], R.IDENTITY_B, atol=1e-10)
    r = O.cg(O.op_diagonal(R.DIAG["diag"]), R.DIAG["b"])
    assert r["converged"] and np.allclose(r["x"], R.DIAG["x"], atol=1e-10)


def test_bicgstab_identity_and_diagonal():
    r = O.bicgstab(O.op_identity(3), R.IDENTITY_B)
    assert r["converged"] and np.allclose(r["x"], R.IDENTITY_B, atol=1e-10)
    r = O.bicgstab(O.op_diagonal(R.DIAG["diag"]), R.DIAG["b"])
    assert r["converged"] and np.allclose(r["x"], R.DIAG["x"], atol=1e-10)


def test_cg_sparse_3x3():
    c = R.SPD3
    a = op_from_triplets(c["rows"], c["cols"], c["data"], (3, 3))
    r = O.cg(a, c["b"])
    assert r["converged"]
    assert np.all(np.abs(a.matvec(r["x"]) - c["b"]) < c["tol"])


def test_bicgstab_non_symmetric():
    c = R.NONSYM3
    a = op_from_triplets(c["rows"], c["cols"], c["data"], (3, 3))
    r = O.bicgstab(a, c["b"])
    assert r["converged"]
    assert np.all(np.abs(a.matvec(r["x"]) - c["b"]) < c["tol"])


def test_cg_2x2():
    c = R.CG_2X2
    a = op_from_triplets(c["rows"], c["cols"], c["data"], (2, 2))
    r = O.cg(a, c["b"])
    assert r["converged"] and np.allclose(r["x"], c["x"], atol=c["tol"])


def test_cg_with_jacobi():
    c = R.CG_JACOBI
    a = op_from_triplets(c["rows"], c["cols"], c["data"], (3, 3))
    r = O.cg(a, c["b"], preconditioner=O.op_jacobi(a))
    assert r["converged"] and r["iterations"] < c["max_iterations"]
    assert np.allclose(a.matvec(r["x"]), c["b"], atol=c["tol"])


def test_jacobi_apply():
    c = R.JACOBI_APPLY
    e = O.Err()
    d = np.asarray(c["diag"])
    h = O.lib().or_op_jacobi_from_diagonal(1, O.p(d), 3, C.byref(e))
    m = O.Op(h, 3)
    assert np.allclose(m.matvec(c["x"]), c["y"], atol=1e-10)
    a = op_from_triplets([0, 1, 2], [0, 1, 2], c["diag"], (3, 3))
    assert np.allclose(O.op_jacobi(a).matvec(c["x"]), c["y"], atol=1e-10)


def test_bicgstab_duplicate_entry_with_jacobi():
    c = R.BICGSTAB_DUP
    a = op_from_triplets(c["rows"], c["cols"], c["data"], c["shape"])
    m = O.op_jacobi(a)
    # the Jacobi preconditioner takes the first duplicate (15), SpMV sums both (16)
    assert np.isclose(m.matvec([0, 0, 0, 1.0])[3], 1.0 / 15.0)
    assert np.isclose(a.matvec([0, 0, 0, 1.0])[3], 16.0)
    r = O.bicgstab(a, c["b"], max_iter=c["max_iter"], rtol=c["rtol"], atol=c["atol"], left=m)
    assert r["converged"] and r["iterations"] < c["max_iterations"]
    assert np.linalg.norm(np.asarray(c["b"]) - a.matvec(r["x"])) < c["resid"]


def test_bicgstab_convection_diffusion():
    c = R.convection_diffusion()
    a = op_from_triplets(c["rows"], c["cols"], c["data"], c["shape"])
    r = O.bicgstab(a, c["b"], max_iter=c["max_iter"], rtol=c["rtol"], atol=c["atol"])
    assert r["converged"]
    assert np.linalg.norm(np.asarray(c["b"]) - a.matvec(r["x"])) < c["resid"]


def test_bicgstab_breakdown():
    c = R.SINGULAR
    a = op_from_triplets(c["rows"], c["cols"], c["data"], c["shape"])
    r = O.bicgstab(a, c["b"])
    assert not r["converged"] and "breakdown" in r["message"]


def test_ic0_simple_and_not_spd():
    c = R.IC0_SPD
    a = O.op_csr(c["indptr"], c["indices"], np.asarray(c["data"]), (3, 3))
    m = O.op_ic0(a)
    assert np.all(np.isfinite(m.matvec(c["b"])))
    c = R.IC0_NOT_SPD
    a = O.op_csr(c["indptr"], c["indices"], np.asarray(c["data"]), (2, 2))
    with pytest.raises(ValueError):
        O.op_ic0(a)


def test_ic0_quirk_factor_matches_restated_formula():
    # For sorted input the off-diagonals of L are A's, and
    # L_ii = sqrt(a_ii - sum_k a_ik^2 / L_kk) (ic.rs:76-104): tridiag(-1, 4, -1)
    c = R.IC0_SPD
    a = O.op_csr(c["indptr"], c["indices"], np.asarray(c["data"]), (3, 3))
    m = O.op_ic0(a)
    nnz = O.lib().or_ic0_nnz(m.h)
    ip = np.empty(4, dtype=np.uint64)
    ix = np.empty(nnz, dtype=np.uint64)
    d = np.empty(nnz)
    O.lib().or_ic0_factor(m.h, O.p(ip), O.p(ix), O.p(d))
    l00 = 2.0
    l11 = np.sqrt(4.0 - 1.0 / l00)
    l22 = np.sqrt(4.0 - 1.0 / l11)
    assert np.allclose(d, [l00, -1.0, l11, -1.0, l22])


def test_ic0_fast_backward_is_bit_identical():
    rng = np.random.default_rng(3)
    n = 60
    a = np.zeros((n, n))
    for i in range(n):
        a[i, i] = 6.0
        for j in rng.choice(n, 3):
            if j != i:
                a[i, j] = a[j, i] = -rng.uniform(0.1, 1.0)
    ip = [0]
    ix, dv = [], []
    for i in range(n):
        for j in range(n):
            if a[i, j] != 0:
                ix.append(j)
                dv.append(a[i, j])
        ip.append(len(ix))
    op = O.op_csr(ip, ix, np.asarray(dv), (n, n))
    slow, fast = O.op_ic0(op, fast=False), O.op_ic0(op, fast=True)
    x = rng.standard_normal(n)
    assert np.array_equal(slow.matvec(x), fast.matvec(x))


def test_construction_errors():
    rc, msg, *_ = csr_new([0, 3], [0, 0], [1.0, 2.0], (3, 3))
    assert rc == 9 and msg == "Value error: Row index out of bounds"
    rc, msg, *_ = csr_new([0, 1], [0, 5], [1.0, 2.0], (3, 3))
    assert rc == 9 and msg == "Value error: Column index out of bounds"
    e = O.Err()
    ip = np.asarray([0, 2, 1], dtype=np.uint64)
    ix = np.asarray([0, 1], dtype=np.uint64)
    assert O.lib().or_csr_matrix_from_raw_check(O.p(ip), 3, O.p(ix), 2, 2, 2, 2, C.byref(e)) == 9
    assert e.msg.decode() == "Value error: Row pointer array must be monotonically increasing"


def test_gmres_solves_small_systems():
    # gmres has no test in the reference crate; check the restatement solves
    c = R.NONSYM3
    a = op_from_triplets(c["rows"], c["cols"], c["data"], (3, 3))
    r = O.gmres(a, c["b"])
    assert r["converged"]
    assert np.all(np.abs(a.matvec(r["x"]) - c["b"]) < 1e-9)
    c = R.convection_diffusion()
    a = op_from_triplets(c["rows"], c["cols"], c["data"], c["shape"])
    r = O.gmres(a, c["b"], restart=4)
    assert r["converged"] and np.linalg.norm(np.asarray(c["b"]) - a.matvec(r["x"])) < 1e-6

