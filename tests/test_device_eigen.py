"""power_iteration and lanczos on the device vs the oracle (eigen.rs:124-494).

The device sums are tree reductions, the oracle's (like the reference's)
sequential folds, so values agree to rounding: eigenvalues, residuals and
vectors within the tolerances below, iteration counts and outcomes exactly
(or within one step where a stopping test compares nearly equal numbers).
Error and panic cases give the same messages.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _lower(ip, ix, v):
    """Lower triangle (col <= row) of a CSR matrix, rows sorted."""
    n = len(ip) - 1
    rows = np.repeat(np.arange(n), np.diff(ip))
    keep = ix <= rows
    lip = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(np.uint64)
    return lip, ix[keep].astype(np.uint64), v[keep]


def _sym(S, ctx, lip, lix, lv, dtype=np.float64):
    n = len(lip) - 1
    return S.sym_csr_matrix(ctx, np.asarray(lv, dtype=dtype), lip, lix, (n, n), dtype=dtype)


REF = (np.array([0, 1, 3, 5], dtype=np.uint64), np.array([0, 0, 1, 1, 2], dtype=np.uint64),
       np.array([2.0, 1.0, 2.0, 3.0, 1.0]))


def _close(a, b, rtol, atol=0.0):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.allclose(a, b, rtol=rtol, atol=atol), (a, b)


def test_power_iteration_matches_oracle(S, ctx):
    rng = np.random.default_rng(4)
    ip, ix, v = S.generate("poisson2d", 20, 20)
    cases = [("ref", REF, None), ("poisson20", _lower(ip, ix, v), rng.standard_normal(400))]
    for name, (lip, lix, lv), x0 in cases:
        a = _sym(S, ctx, lip, lix, lv)
        for normalize in (True, False):
            kw = dict(max_iter=60 if not normalize else 300, tol=1e-9, normalize=normalize, initial_guess=x0)
            d = S.power_iteration(a, **kw)
            o = O.power_iteration(lip, lix, lv, **kw)
            assert d.converged == o["converged"], name
            assert abs(d.iterations - o["iterations"]) <= 1, (name, d.iterations, o["iterations"])
            _close(d.eigenvalues, o["eigenvalues"], 1e-9)
            if d.iterations == o["iterations"] and normalize:
                _close(d.eigenvectors, o["eigenvectors"], 1e-7, 1e-12)
            # the residual is ||Ax - lambda x|| of the returned pair
            x = d.eigenvectors[:, 0]
            r = a.matvec(x) - d.eigenvalues[0] * x
            assert abs(np.linalg.norm(r) - d.residuals[0]) <= 1e-9 * max(1.0, np.linalg.norm(a.matvec(x)))


def test_power_iteration_fp32(S, ctx):
    lip, lix, lv = REF
    a = _sym(S, ctx, lip, lix, lv, np.float32)
    d = S.power_iteration(a, tol=1e-5)
    o = O.power_iteration(lip, lix, lv.astype(np.float32), tol=1e-5)
    assert d.eigenvalues.dtype == np.float32 and d.converged == o["converged"]
    _close(d.eigenvalues, o["eigenvalues"], 1e-5)


def test_lanczos_closed_forms_match_oracle(S, ctx):
    rng = np.random.default_rng(9)
    ip, ix, v = S.generate("poisson2d", 12, 12)
    pois = _lower(ip, ix, v)
    x0 = rng.standard_normal(144)
    for (lip, lix, lv), v0 in ((REF, None), (pois, x0)):
        a = _sym(S, ctx, lip, lix, lv)
        for sub in (1, 2, 3):
            for num in range(1, sub + 1):
                for vecs in (True, False):
                    kw = dict(max_iter=100, max_subspace_size=sub, tol=1e-10, num_eigenvalues=num,
                              compute_eigenvectors=vecs, initial_guess=v0)
                    d = S.lanczos(a, **kw)
                    o = O.lanczos(lip, lix, lv, **kw)
                    assert (d.iterations, d.converged) == (o["iterations"], o["converged"]), kw
                    _close(d.eigenvalues, o["eigenvalues"], 1e-8, 1e-10)
                    _close(d.residuals, o["residuals"], 1e-6, 1e-9)
                    if vecs:
                        _close(d.eigenvectors, o["eigenvectors"], 1e-7, 1e-9)
                    else:
                        assert d.eigenvectors is None


def test_lanczos_errors_match_oracle(S, ctx):
    ip, ix, v = S.generate("poisson2d", 12, 12)
    lip, lix, lv = _lower(ip, ix, v)
    a = _sym(S, ctx, lip, lix, lv)
    # four or more steps: the reference's QL sweep never converges
    with pytest.raises(S.SparseError, match="QL algorithm did not converge") as e:
        S.lanczos(a, max_subspace_size=6, num_eigenvalues=2)
    with pytest.raises(O.OracleError, match="QL algorithm did not converge"):
        O.lanczos(lip, lix, lv, max_subspace_size=6, num_eigenvalues=2)
    assert e.value.code == 13
    # beta_1 = 0 (e_0 is an eigenvector of a diagonal matrix): one alpha,
    # and a second requested eigenvalue indexes past the list (a panic)
    n = 40
    dip, dix, dv = np.arange(n + 1, dtype=np.uint64), np.arange(n, dtype=np.uint64), np.linspace(1.0, 2.0, n)
    dg = _sym(S, ctx, dip, dix, dv)
    with pytest.raises(S.SparseError, match="panic"):
        S.lanczos(dg, max_subspace_size=5, num_eigenvalues=2)
    with pytest.raises(O.OracleError, match="panic"):
        O.lanczos(dip, dix, dv, max_subspace_size=5, num_eigenvalues=2)
    r = S.lanczos(dg, max_subspace_size=5, num_eigenvalues=1)
    assert r.eigenvalues[0] == 1.0 and r.iterations == 1 and r.residuals[0] == 0.0
    with pytest.raises(S.SparseError, match="capacity overflow"):
        S.lanczos(dg, max_subspace_size=0)
    with pytest.raises(S.SparseError, match="Dimension mismatch: expected 40, found 3"):
        S.lanczos(dg, initial_guess=[1.0, 2.0, 3.0])
    with pytest.raises(S.SparseError, match="Dimension mismatch: expected 40, found 2"):
        S.power_iteration(dg, initial_guess=[1.0, 2.0])
    csr = S.csr_from_arrays(ctx, ip, ix, v, (144, 144))
    with pytest.raises(S.SparseError, match="not a symmetric CSR operator"):
        S.power_iteration(csr)


def test_large_power_iteration(S, ctx):
    # a 256^2 Laplacian: the device path at size, against the known top
    # eigenvalue 8 sin^2(pi 256 / (2 * 257)) (within the iteration's error)
    m = 256
    ip, ix, v = S.generate("poisson2d", m, m)
    lip, lix, lv = _lower(ip, ix, v)
    a = _sym(S, ctx, lip, lix, lv)
    x0 = np.random.default_rng(1).standard_normal(m * m)
    d = S.power_iteration(a, max_iter=2000, tol=1e-9, initial_guess=x0)
    top = 8.0 * np.sin(np.pi * m / (2.0 * (m + 1))) ** 2
    assert abs(d.eigenvalues[0] - top) < 1e-3 * top
    x = d.eigenvectors[:, 0]
    assert abs(np.linalg.norm(x) - 1.0) < 1e-9


def test_lanczos_odd_sizes_on_the_diagonal_layout(S, ctx):
    # odd n: the basis vectors sit one padded stride apart, so every SpMV
    # operand is aligned for the diagonal layout's vector loads
    rng = np.random.default_rng(5)
    ip, ix, v = S.generate("poisson2d", 21, 19)
    cases = [(_lower(ip, ix, v), rng.standard_normal(399)),
             ((np.array([0, 1, 3, 5, 7, 9], dtype=np.uint64), np.array([0, 0, 1, 1, 2, 2, 3, 3, 4], dtype=np.uint64),
               np.array([4.0, -1, 4, -1, 4, -1, 4, -1, 4])), None)]
    for (lip, lix, lv), v0 in cases:
        a = _sym(S, ctx, lip, lix, lv)
        assert S.spmv_kernel(a).startswith("spmv_dia")
        kw = dict(max_iter=100, max_subspace_size=3, tol=1e-10, num_eigenvalues=2, compute_eigenvectors=True,
                  initial_guess=v0)
        d = S.lanczos(a, **kw)
        o = O.lanczos(lip, lix, lv, **kw)
        assert (d.iterations, d.converged) == (o["iterations"], o["converged"])
        _close(d.eigenvalues, o["eigenvalues"], 1e-8, 1e-10)
        _close(d.eigenvectors, o["eigenvectors"], 1e-7, 1e-9)
        a.close()
