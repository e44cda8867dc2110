"""The oracle's ILU(0) and SSOR (preconditioners.rs:94-399).

The reference has no test of either; these pin the restatement on known
answers instead: ILU(0) of a tridiagonal matrix is its exact LU factorisation
(no fill-in is dropped), so M^-1 A = I; SSOR with omega = 1 on a diagonal
matrix applies x / d; a hand-worked 2 x 2 SSOR product; and the reference's
error messages.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O
from tests.test_oracle_reference import csr_new


def csr_op(rows, cols, data, shape):
    rc, _, ip, ix, d = csr_new(rows, cols, data, shape)
    assert rc == 0
    return O.op_csr(ip, ix, d, shape)


def tridiag(n, rng):
    rows, cols, data = [], [], []
    for i in range(n):
        for j in (i - 1, i, i + 1):
            if 0 <= j < n:
                rows.append(i); cols.append(j)
                data.append(4.0 + rng.uniform() if i == j else rng.uniform(-1.0, 1.0))
    return rows, cols, data


def test_ilu0_of_tridiagonal_is_exact():
    rng = np.random.default_rng(0)
    n = 30
    rows, cols, data = tridiag(n, rng)
    a = csr_op(rows, cols, data, (n, n))
    m = O.op_ilu0(a)
    dense = np.zeros((n, n))
    for r, c, v in zip(rows, cols, data):
        dense[r, c] += v
    x = rng.standard_normal(n)
    assert np.allclose(m.matvec(dense @ x), x, rtol=1e-12, atol=1e-12)


def test_ssor_known_answers():
    # omega = 1, diagonal matrix: y = x / d, z = y * d = x, w = z / d
    a = csr_op([0, 1, 2], [0, 1, 2], [2.0, 4.0, 8.0], (3, 3))
    m = O.op_ssor(a, 1.0)
    assert np.allclose(m.matvec([2.0, 4.0, 8.0]), [1.0, 1.0, 1.0])
    # [[2, 1], [1, 2]], omega = 1, x = [1, 1]:
    # y0 = 1/2, y1 = (1 - 1/2)/2 = 1/4; z = [1, 1/2]; w1 = (1/2)/2 = 1/4, w0 = (1 - 1/4)/2 = 3/8
    a = csr_op([0, 0, 1, 1], [0, 1, 0, 1], [2.0, 1.0, 1.0, 2.0], (2, 2))
    assert np.allclose(O.op_ssor(a, 1.0).matvec([1.0, 1.0]), [0.375, 0.25])
    # omega = 0.5: y0 = 1/2, y1 = (1 - 0.5 * 1/2) / 2 = 3/8; z = [1, 3/4];
    # w1 = 3/8, w0 = (1 - 0.5 * 3/8) / 2 = 13/32
    assert np.allclose(O.op_ssor(a, 0.5).matvec([1.0, 1.0]), [13 / 32, 3 / 8])


def test_errors():
    a = csr_op([0, 1], [0, 1], [1.0, 1.0], (2, 2))
    for om in (0.0, 2.0, -1.0):
        with pytest.raises(ValueError, match="Relaxation parameter omega must be in \\(0, 2\\)"):
            O.op_ssor(a, om)
    z = csr_op([0, 1], [0, 0], [1.0, 1.0], (2, 2))
    with pytest.raises(ValueError, match="Zero diagonal element at position 1"):
        O.op_ssor(z, 1.0)
    with pytest.raises(ValueError, match="Missing diagonal element at row 1"):
        O.op_ilu0(z)
    p = csr_op([0, 0, 1, 1], [0, 1, 0, 1], [1.0, 1.0, 1.0, 1.0], (2, 2))
    with pytest.raises(ValueError, match="Zero pivot at position 1"):
        O.op_ilu0(p)


def test_ilu0_improves_cg_free_solvers():
    # ILU(0)-preconditioned gmres needs fewer iterations than plain gmres
    n = 12
    rows, cols, data = [], [], []
    for i in range(n):
        for j in range(n):
            k = i * n + j
            rows.append(k); cols.append(k); data.append(4.0)
            for di, dj, v in ((-1, 0, -1.2), (1, 0, -0.8), (0, -1, -1.0), (0, 1, -1.0)):
                ii, jj = i + di, j + dj
                if 0 <= ii < n and 0 <= jj < n:
                    rows.append(k); cols.append(ii * n + jj); data.append(v)
    a = csr_op(rows, cols, data, (n * n, n * n))
    b = np.ones(n * n)
    r0 = O.gmres(a, b, rtol=1e-10)
    r1 = O.gmres(a, b, rtol=1e-10, preconditioner=O.op_ilu0(a))
    r2 = O.gmres(a, b, rtol=1e-10, preconditioner=O.op_ssor(a, 1.2))
    assert r0["converged"] and r1["converged"] and r2["converged"]
    assert r1["iterations"] < r0["iterations"] and r2["iterations"] < r0["iterations"]
