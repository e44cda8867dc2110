"""The oracle's restatement of linalg/eigen.rs against the reference's tests.

eigen.rs:1068-1112 (tridiagonal 2x2 and cubic solver tests) pass as
written.  eigen.rs:996-1066 assert that the test matrix [[2,1,0],[1,2,3],
[0,3,1]] has eigenvalues 5, 1 and -1; it has 4.7577, 1.9009 and -1.6586,
so those two tests fail in the reference itself.  Here power_iteration is
checked against the true largest eigenvalue (with normalize it is a plain
power iteration; without, it returns x.Ax / ||Ax||^2, i.e. 1 / lambda),
and lanczos against what the reference's loops compute: the
first beta is kept for every step, solve_cubic's trigonometric branch
takes acos(+b), and with four or more Lanczos steps the QL sweep, which
never updates e[0], fails with "QL algorithm did not converge".
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

IP = [0, 1, 3, 5]
IX = [0, 0, 1, 1, 2]
DATA = np.array([2.0, 1.0, 2.0, 3.0, 1.0])
DENSE = np.array([[2.0, 1.0, 0.0], [1.0, 2.0, 3.0], [0.0, 3.0, 1.0]])


def test_cubic_solver_reference_cases():
    # eigen.rs:1087-1111
    assert np.allclose(sorted(O.solve_cubic(-6.0, 11.0, -6.0)), [1.0, 2.0, 3.0], atol=1e-8)
    assert np.allclose(sorted(O.solve_cubic(0.0, -4.0, 0.0)), [-2.0, 0.0, 2.0], atol=1e-8)
    # one real root (discriminant 4a^3 + 27b^2 > 0): the reference's Cardano
    # step takes (-b +- sqrt(disc) / 2) / 2 where the formula has
    # -b/2 +- sqrt(disc / 108), so x^3 + x + 1 gets -0.2742 (its root is -0.6823)
    r = O.solve_cubic(0.0, 1.0, 1.0)
    c1, c2 = (-1.0 + np.sqrt(31.0) * 0.5) / 2.0, (-1.0 - np.sqrt(31.0) * 0.5) / 2.0
    want = np.cbrt(c1) + np.cbrt(c2)
    assert len(r) == 1 and abs(r[0] - want) < 1e-12 and abs(r[0] + 0.6823278038280193) > 0.1
    # with b != 0 the trigonometric branch returns roots that are not those
    # of the cubic (acos(+b) where the formula needs acos(-b)); the sum of
    # the roots is still -p
    r = O.solve_cubic(70.0, -146.0, -70.0)
    assert abs(sum(r) + 70.0) < 1e-9
    true = np.roots([1.0, 70.0, -146.0, -70.0])
    assert not np.allclose(sorted(r), sorted(true.real))


def test_tridiagonal_2x2_reference_case():
    # eigen.rs:1068-1085
    vals, vecs = O.tridiag_eig([2.0, 1.0], [1.0], 2)
    assert np.allclose(vals, [2.618033988749895, 0.381966011250105], atol=1e-8)
    for v in vecs:
        assert abs(np.linalg.norm(v) - 1.0) < 1e-8


def test_tridiagonal_small_and_ql_paths():
    vals, vecs = O.tridiag_eig([3.0], [], 2)
    assert list(vals) == [3.0] and len(vecs) == 1
    vals, _ = O.tridiag_eig([2.0, 1.0], [0.0], 1)
    assert list(vals) == [2.0]
    # b = 0 in the depressed cubic: the 3x3 closed form is right
    vals, vecs = O.tridiag_eig([1.0, 1.0, 1.0], [1.0, 1.0], 3)
    assert np.allclose(vals, [1 + np.sqrt(2), 1.0, 1 - np.sqrt(2)], atol=1e-12)
    # four or more rows: the QL sweep never touches e[0]
    with pytest.raises(O.OracleError, match="QL algorithm did not converge"):
        O.tridiag_eig([2.0, 1.0, 3.0, 4.0], [1.0, 1.0, 1.0], 2)
    # ... unless e[0] is already negligible
    vals, _ = O.tridiag_eig([2.0, 1.0, 3.0, 4.0], [0.0, 0.0, 0.0], 4)
    assert list(vals) == [4.0, 3.0, 2.0, 1.0]
    with pytest.raises(O.OracleError, match="Empty tridiagonal matrix"):
        O.tridiag_eig([], [], 1)


def test_power_iteration_on_the_reference_matrix():
    r = O.power_iteration(IP, IX, DATA, max_iter=100, tol=1e-10)
    top = np.linalg.eigvalsh(DENSE)[-1]
    assert r["converged"] and abs(r["eigenvalues"][0] - top) < 1e-8
    v = r["eigenvectors"][:, 0]
    assert abs(np.linalg.norm(v) - 1.0) < 1e-8
    assert np.allclose(O.sym_matvec(IP, IX, DATA, v), top * v, atol=1e-4)
    assert abs(r["residuals"][0] - np.linalg.norm(DENSE @ v - r["eigenvalues"][0] * v)) < 1e-12
    # not normalising: lambda = x.(Ax) / ||Ax||^2 (eigen.rs:225-234 divides by
    # the norm of the new x = Ax), which tends to 1 / lambda_max
    r = O.power_iteration(IP, IX, DATA, max_iter=200, tol=1e-10, normalize=False)
    assert r["converged"] and abs(r["eigenvalues"][0] - 1.0 / top) < 1e-8
    with pytest.raises(O.OracleError, match="Dimension mismatch: expected 3, found 2"):
        O.power_iteration(IP, IX, DATA, initial_guess=[1.0, 2.0])


def test_lanczos_on_the_reference_matrix():
    r = O.lanczos(IP, IX, DATA, max_iter=100, max_subspace_size=3, tol=1e-10, num_eigenvalues=3)
    # the tridiagonal matrix the reference builds: alpha = [2, 0, -72],
    # beta = [1, 1] (beta_1 kept), and its closed-form "roots"
    vals, _ = O.tridiag_eig([2.0, 0.0, -72.0], [1.0, 1.0], 3)
    assert np.allclose(r["eigenvalues"], vals, rtol=1e-12)
    assert r["iterations"] == 3 and not r["converged"]
    assert r["eigenvectors"].shape == (3, 3)
    # two steps: the 2x2 closed form
    r = O.lanczos(IP, IX, DATA, max_subspace_size=2, num_eigenvalues=2)
    vals, _ = O.tridiag_eig([2.0, 0.0], [1.0], 2)
    assert np.allclose(r["eigenvalues"], vals, rtol=1e-12)


def test_lanczos_ql_failure_and_panics():
    n = 30
    ip = np.arange(n + 1)
    ix = np.arange(n)
    d = np.linspace(1.0, 3.0, n)
    lower = _path_lower(n)
    with pytest.raises(O.OracleError, match="QL algorithm did not converge"):
        O.lanczos(*lower, max_subspace_size=6, num_eigenvalues=2)
    # e_0 is an eigenvector of a diagonal matrix: beta_1 = 0, one alpha, and
    # two requested eigenvalues index past the one the closed form returns
    with pytest.raises(O.OracleError, match="panic"):
        O.lanczos(ip, ix, d, max_subspace_size=5, num_eigenvalues=2)
    r = O.lanczos(ip, ix, d, max_subspace_size=5, num_eigenvalues=1)
    assert r["eigenvalues"][0] == 1.0 and r["iterations"] == 1
    with pytest.raises(O.OracleError, match="capacity overflow"):
        O.lanczos(ip, ix, d, max_subspace_size=0)


def _path_lower(n, diag=4.0):
    """Lower triangle of tridiag(-1, diag, -1)."""
    ip = [0]
    ix, dv = [], []
    for i in range(n):
        if i:
            ix.append(i - 1)
            dv.append(-1.0)
        ix.append(i)
        dv.append(diag)
        ip.append(len(ix))
    return np.array(ip), np.array(ix), np.array(dv)
