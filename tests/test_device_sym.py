"""Symmetric CSR (lower triangle stored) on the device vs the oracle.

The reference's known answers (sym_csr.rs:498-593, sym_ops.rs:348-459,
test_dimension_mismatch.rs:5-33) go through the device API; random lower
triangles with unsorted columns, duplicates and empty rows are compared with
the oracle bit for bit (matvec, get, nnz, trace, quadratic form, rank-1
update, from_csr), under every SpMV kernel choice.  The half-storage product
(SX_SPMV_SYM_HALF, atomic scatter) is held to a few ulp of sum |a_ij x_j|.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle_ffi as O
from tests.test_oracle_sym import DATA, INDICES, INDPTR, VALIDATION_CASES, random_lower

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _ctx_with(S, env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return S.Context(0)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


def test_reference_creation(S, ctx):
    m = S.sym_csr_matrix(ctx, DATA, INDPTR, INDICES, (3, 3))
    assert m.shape == (3, 3)
    assert m.nnz_stored() == 5 and m.nnz == 7
    expect = {(0, 0): 2.0, (0, 1): 1.0, (1, 0): 1.0, (1, 1): 2.0, (1, 2): 3.0, (2, 1): 3.0,
              (0, 2): 0.0, (2, 0): 0.0, (2, 2): 1.0, (3, 0): 0.0, (0, 9): 0.0}
    for (i, j), v in expect.items():
        assert m.get(i, j) == v, (i, j)
    ip, ix, dv = m.to_arrays()
    assert list(ip) == list(INDPTR) and list(ix) == list(INDICES) and list(dv) == list(DATA)
    assert m.has_adjoint


def test_reference_matvec_quadratic_trace(S, ctx):
    x = np.array([1.0, 2.0, 3.0])
    for dt in (np.float64, np.float32):
        m = S.sym_csr_matrix(ctx, DATA, INDPTR, INDICES, (3, 3), dtype=dt)
        y = S.sym_csr_matvec(m, x)
        assert y.dtype == dt and list(y) == [4.0, 14.0, 9.0]
        assert list(m.rmatvec(x)) == [4.0, 14.0, 9.0]
        assert S.sym_csr_quadratic_form(m, x) == 59.0
        assert S.sym_csr_trace(m) == 5.0
    with pytest.raises(S.SparseError, match=r"Dimension mismatch: expected 3, found 2"):
        m.matvec(np.ones(2))
    with pytest.raises(S.SparseError, match=r"Dimension mismatch: expected 3, found 4"):
        S.sym_csr_quadratic_form(m, np.ones(4))


def test_reference_rank1_update(S, ctx):
    m = S.sym_csr_matrix(ctx, DATA, INDPTR, INDICES, (3, 3))
    S.sym_csr_rank1_update(m, np.array([1.0, 0.0, 0.0]), 3.0)
    assert m.get(0, 0) == 5.0
    assert (m.get(0, 1), m.get(1, 1), m.get(1, 2), m.get(2, 2)) == (1.0, 2.0, 3.0, 1.0)
    assert list(S.sym_csr_matvec(m, np.array([1.0, 2.0, 3.0]))) == [7.0, 14.0, 9.0]
    with pytest.raises(S.SparseError, match=r"Dimension mismatch: expected 3, found 1"):
        S.sym_csr_rank1_update(m, np.ones(1), 1.0)


def test_reference_from_and_to_csr(S, ctx):
    rows, cols = [0, 0, 1, 1, 1, 2, 2], [0, 1, 0, 1, 2, 1, 2]
    data = [2.0, 1.0, 1.0, 2.0, 3.0, 3.0, 1.0]
    csr = S.csr_matrix(ctx, data, rows, cols, (3, 3))
    m = S.sym_csr_from_csr(csr)
    assert m.shape == (3, 3)
    dense = m.to_csr().to_dense()
    assert dense.tolist() == [[2.0, 1.0, 0.0], [1.0, 2.0, 3.0], [0.0, 3.0, 1.0]]
    assert m.to_dense().tolist() == dense.tolist()
    full = S.sym_csr_matrix(ctx, DATA, INDPTR, INDICES, (3, 3)).to_csr()
    for (i, j), v in {(0, 0): 2.0, (0, 1): 1.0, (1, 0): 1.0, (1, 1): 2.0, (1, 2): 3.0, (2, 1): 3.0,
                      (2, 2): 1.0, (0, 2): 0.0, (2, 0): 0.0}.items():
        assert full.get(i, j) == v
    bad = S.csr_matrix(ctx, data, [0, 0, 1, 1, 2, 2, 2], [0, 1, 0, 1, 0, 1, 2], (3, 3))
    with pytest.raises(S.SparseError, match="Value error: Matrix must be symmetric to convert to SymCSR format"):
        S.sym_csr_from_csr(bad)
    rect = S.csr_matrix(ctx, [1.0], [0], [0], (2, 3))
    with pytest.raises(S.SparseError, match="Value error: Symmetric matrix must be square"):
        S.sym_csr_from_csr(rect)


@pytest.mark.parametrize("case", range(len(VALIDATION_CASES)))
def test_validation_matches_oracle(S, ctx, case):
    (data_len, ip, ix, shape), msg = VALIDATION_CASES[case]
    with pytest.raises(S.SparseError) as e:
        S.sym_csr_matrix(ctx, np.ones(data_len), ip, ix, shape)
    assert str(e.value) == msg
    assert O.sym_check(data_len, ip, ix, shape)[1] == msg


@pytest.mark.parametrize("n", [1, 7, 1000, 20000])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_random_bit_exact(S, ctx, n, dt):
    rng = np.random.default_rng(n * 3 + (dt == np.float32))
    ip, ix, dv = random_lower(rng, n, max_len=12)
    dv = dv.astype(dt)
    m = S.sym_csr_matrix(ctx, dv, ip, ix, (n, n), dtype=dt)
    x = rng.standard_normal(n).astype(dt)
    y = S.sym_csr_matvec(m, x)
    ref = O.sym_matvec(ip, ix, dv, x)
    assert np.array_equal(_bits(y), _bits(ref))
    assert m.nnz == O.sym_nnz(ip, ix) and m.nnz_stored() == len(ix)
    q = S.sym_csr_quadratic_form(m, x)
    assert _bits(np.array([q], dtype=dt))[0] == _bits(np.array([O.sym_quadratic_form(ip, ix, dv, x)], dtype=dt))[0]
    t = S.sym_csr_trace(m)
    assert _bits(np.array([t], dtype=dt))[0] == _bits(np.array([O.sym_trace(ip, ix, dv)], dtype=dt))[0]
    for _ in range(20):
        i, j = (int(v) for v in rng.integers(0, n + 1, 2))
        assert m.get(i, j) == dt(O.sym_get(ip, ix, dv.astype(np.float64), i, j))
    rip, rix, rdv = m.to_arrays()
    assert np.array_equal(rip, ip) and np.array_equal(rix, ix) and np.array_equal(_bits(rdv), _bits(dv))


def _lower_of(ip, ix, dv):
    n = len(ip) - 1
    rows = np.repeat(np.arange(n), np.diff(ip))
    keep = ix <= rows
    lens = np.bincount(rows[keep], minlength=n)
    lip = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    return lip, ix[keep].astype(np.uint64), dv[keep]


@pytest.mark.parametrize("env", [{}, {"SX_DIA_ND6": "0"}, {"SX_DIA": "0"}, {"SX_DIA": "0", "SX_WIN": "2"}, {"SX_DIA": "0", "SX_SHORT": "2"},
                                 {"SX_DIA": "0", "SX_WIN": "0", "SX_SHORT": "0"}])
@pytest.mark.parametrize("kind", ["laplace3d", "powerlaw"])
def test_kernel_choices_bit_exact(S, env, kind):
    if kind == "laplace3d":
        ip, ix, dv = S.generate("laplace3d", 48, 48, 48)
    else:
        ip, ix, dv = S.generate("powerlaw", 60000, seed=3, param0=16.0, param1=2048.0)
    lip, lix, ldv = _lower_of(ip, ix, dv)
    n = len(lip) - 1
    c = _ctx_with(S, env)
    try:
        rng = np.random.default_rng(5)
        for dt in (np.float64, np.float32):
            m = S.sym_csr_matrix(c, ldv.astype(dt), lip, lix, (n, n), dtype=dt)
            x = rng.standard_normal(n).astype(dt)
            y = S.sym_csr_matvec(m, x)
            assert np.array_equal(_bits(y), _bits(O.sym_matvec(lip, lix, ldv.astype(dt), x))), (env, dt)
            m.close()
    finally:
        c.close()


def test_from_csr_laplacian_bit_exact(S, ctx):
    ip, ix, dv = S.generate("laplace3d", 64, 64, 64)
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, dv, (n, n))
    m = S.sym_csr_from_csr(a)
    (lip, lix, ldv), err = O.sym_from_csr(ip.astype(np.uint64), ix.astype(np.uint64), dv, (n, n))
    assert err is None
    rip, rix, rdv = m.to_arrays()
    assert np.array_equal(rip, lip) and np.array_equal(rix, lix) and np.array_equal(_bits(rdv), _bits(ldv))
    x = np.random.default_rng(1).standard_normal(n)
    y = m.matvec(x)
    assert np.array_equal(_bits(y), _bits(O.sym_matvec(lip, lix, ldv, x)))
    # the full CSR product agrees to rounding (different summation order)
    assert np.allclose(y, a.matvec(x), rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("dup", [False, True])
def test_from_csr_random(S, ctx, dup):
    # with duplicate positions, is_symmetric compares each copy with the
    # first copy of its mirror (CsrMatrix::get), so both sides refuse
    rng = np.random.default_rng(11 + dup)
    n = 3000
    lip, lix, ldv = random_lower(rng, n, max_len=6, dup=dup)
    full = S.sym_csr_matrix(ctx, ldv, lip, lix, (n, n)).to_csr()
    fip, fix, fdv = full.to_arrays()
    res, err = O.sym_from_csr(fip, fix, fdv, (n, n))
    if err is not None:
        assert dup
        with pytest.raises(S.SparseError) as e:
            S.sym_csr_from_csr(full)
        assert str(e.value) == err
        return
    m = S.sym_csr_from_csr(full)
    oip, oix, odv = res
    rip, rix, rdv = m.to_arrays()
    assert np.array_equal(rip, oip) and np.array_equal(rix, oix) and np.array_equal(_bits(rdv), _bits(odv))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_rank1_update_bit_exact(S, ctx, dt):
    rng = np.random.default_rng(21)
    n = 700
    ip, ix, dv = random_lower(rng, n, max_len=5)
    dv = dv.astype(dt)
    x = rng.standard_normal(n).astype(dt)
    x[rng.integers(0, n, 100)] = 0.0
    alpha = dt(-0.75)
    m = S.sym_csr_matrix(ctx, dv, ip, ix, (n, n), dtype=dt)
    S.sym_csr_rank1_update(m, x, float(alpha))
    oip, oix, odv = O.sym_rank1_update(ip, ix, dv, x, alpha)
    rip, rix, rdv = m.to_arrays()
    assert np.array_equal(rip, oip) and np.array_equal(rix, oix) and np.array_equal(_bits(rdv), _bits(odv))
    z = rng.standard_normal(n).astype(dt)
    assert np.array_equal(_bits(m.matvec(z)), _bits(O.sym_matvec(oip, oix, odv, z)))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_half_storage_product(S, ctx, dt):
    import torch

    L = S.sparse.L
    ip, ix, dv = S.generate("laplace3d", 40, 40, 40)
    lip, lix, ldv = _lower_of(ip, ix, dv)
    n = len(lip) - 1
    ldv = ldv.astype(dt)
    m = S.sym_csr_matrix(ctx, ldv, lip, lix, (n, n), dtype=dt)
    assert S.spmv_kernel(m, exact=False, sym_half=True) == "k_sym_half"
    assert S.spmv_kernel(m, exact=True, sym_half=True) != "k_sym_half"
    x = np.random.default_rng(2).standard_normal(n).astype(dt)
    tdt = torch.float64 if dt == np.float64 else torch.float32
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(n, dtype=tdt, device="cuda")
    torch.cuda.synchronize()
    S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, m.handle, C.c_void_p(xd.data_ptr()),
                                     C.c_void_p(yd.data_ptr()), L.SX_SPMV_SYM_HALF))
    ctx.synchronize()
    y = yd.cpu().numpy()
    ref = O.sym_matvec(lip, lix, ldv, x)
    bound = O.sym_matvec(lip, lix, np.abs(ldv), np.abs(x))
    eps = np.finfo(dt).eps
    assert np.all(np.abs(y.astype(np.float64) - ref) <= 16 * eps * bound.astype(np.float64) + 1e-300)


def test_cg_on_symmetric_operator(S, ctx):
    ip, ix, dv = S.generate("poisson2d", 96, 96)
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, dv, (n, n))
    m = S.sym_csr_from_csr(a)
    b = S.rhs_normal(3, n)
    r_full = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0)
    r_sym = S.cg(m, b, max_iter=2000, rtol=1e-10, atol=0.0)
    assert r_full.converged and r_sym.converged
    assert abs(r_full.iterations - r_sym.iterations) <= 3
    assert np.linalg.norm(r_sym.x - r_full.x) <= 1e-8 * np.linalg.norm(r_full.x)
    assert S.true_rel_residual(a, b, r_sym.x) <= 1e-9
