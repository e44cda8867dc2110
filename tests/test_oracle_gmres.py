"""gmres known answers for the oracle (CPU).

The reference crate has no gmres test, so the oracle's restatement of
gmres (iterative.rs:641-816) is pinned here on the mathematics of GMRES and
on the conventions that the reference's loop sets:
- after k Arnoldi steps of one cycle, x_k minimises the left-preconditioned
  residual ||M (b - A x)|| over x0 + K_k(M A, M r0) (checked against a
  least-squares solve on an orthonormal Krylov basis built in numpy);
- a restarted run is a sequence of such minimisations, each cycle starting
  from the previous cycle's x, with restart = min(restart, n);
- the tolerance is max(atol, rtol ||b||) with the unpreconditioned b, and
  the reported residual is ||M (b - A x)||, recomputed after each cycle;
- the breakdown test is absolute (h < 10 eps, iterative.rs:727): on a 6 x 6
  matrix with O(1e3) entries the sixth step counts and solves exactly; the
  same matrix scaled to O(1e-6) drops its sixth column, so the cycle ends
  after five steps and the next cycle starts from that iterate;
- a cycle that cannot advance (restart = 0, or A r0 parallel to r0), which
  the reference's loop repeats forever, ends with an error instead.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O


def _matrix(scale=1.0, n=6, seed=3):
    rng = np.random.default_rng(seed)
    a = (4.0 * np.eye(n) + 0.6 * rng.standard_normal((n, n))) * scale
    b = rng.standard_normal(n)
    return a, b


def _op(a):
    n = a.shape[0]
    ip = np.arange(0, n * n + 1, n, dtype=np.int64)
    ix = np.tile(np.arange(n, dtype=np.int64), n)
    return O.op_csr(ip, ix, a.ravel().copy(), (n, n))


def _krylov_min(a, m, b, x0, k):
    """x0 + argmin over K_k(M A, M r0) of ||M (b - A x)||."""
    r0 = m @ (b - a @ x0)
    q = [r0 / np.linalg.norm(r0)]
    for _ in range(k - 1):
        w = m @ (a @ q[-1])
        for _ in range(2):  # orthogonalised twice
            for v in q:
                w = w - (v @ w) * v
        q.append(w / np.linalg.norm(w))
    basis = np.stack(q, 1)
    y = np.linalg.lstsq(m @ a @ basis, r0, rcond=None)[0]
    return x0 + basis @ y


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_cycle_minimises_over_the_krylov_space(k):
    a, b = _matrix()
    r = O.gmres(_op(a), b, max_iter=k, restart=30, rtol=1e-14, atol=0.0)
    assert r["iterations"] == k and not r["converged"]
    ref = _krylov_min(a, np.eye(6), b, np.zeros(6), k)
    assert np.linalg.norm(r["x"] - ref) <= 1e-11 * np.linalg.norm(ref)
    assert r["residual_norm"] == pytest.approx(np.linalg.norm(b - a @ r["x"]), rel=1e-12)


def test_initial_guess_shifts_the_krylov_space():
    a, b = _matrix()
    x0 = np.linspace(-1.0, 1.0, 6)
    r = O.gmres(_op(a), b, max_iter=3, restart=30, rtol=1e-14, atol=0.0, x0=x0)
    ref = _krylov_min(a, np.eye(6), b, x0, 3)
    assert r["iterations"] == 3
    assert np.linalg.norm(r["x"] - ref) <= 1e-11 * np.linalg.norm(ref)


def test_single_precision_follows_the_same_minimisation():
    a, b = _matrix()
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    n = 6
    ip = np.arange(0, n * n + 1, n, dtype=np.int64)
    ix = np.tile(np.arange(n, dtype=np.int32), n)
    op = O.op_csr_i32(ip, ix, a32.ravel().copy(), (n, n), f64=False)
    r = O.gmres(op, b32, max_iter=3, restart=30, rtol=1e-7, atol=0.0)
    ref = _krylov_min(a32.astype(np.float64), np.eye(6), b32.astype(np.float64), np.zeros(6), 3)
    assert r["x"].dtype == np.float32 and r["iterations"] == 3
    assert np.linalg.norm(r["x"] - ref) <= 1e-5 * np.linalg.norm(ref)


def test_restarted_cycles_chain_minimisations():
    a, b = _matrix()
    r = O.gmres(_op(a), b, max_iter=5, restart=2, rtol=1e-14, atol=0.0)
    x = np.zeros(6)
    for k in (2, 2, 1):  # two full cycles, then one step of the third (max_iter)
        x = _krylov_min(a, np.eye(6), b, x, k)
    assert r["iterations"] == 5
    assert np.linalg.norm(r["x"] - x) <= 1e-11 * np.linalg.norm(x)


def test_left_preconditioner_minimises_the_preconditioned_residual():
    a, b = _matrix()
    op = _op(a)
    m = np.diag(1.0 / np.diag(a))
    r = O.gmres(op, b, max_iter=3, restart=30, rtol=1e-14, atol=0.0, preconditioner=O.op_jacobi(op))
    ref = _krylov_min(a, m, b, np.zeros(6), 3)
    assert r["iterations"] == 3
    assert np.linalg.norm(r["x"] - ref) <= 1e-11 * np.linalg.norm(ref)
    assert r["residual_norm"] == pytest.approx(np.linalg.norm(m @ (b - a @ r["x"])), rel=1e-12)


def test_tolerance_uses_the_unpreconditioned_rhs():
    # M = 1000 I: the preconditioned residual is 1000x the true one, and
    # the loop stops on ||M r|| <= rtol ||b||, i.e. ||r|| <= 1e-3 rtol ||b||
    a, b = _matrix()
    op = _op(a)
    rtol = 1e-6
    r = O.gmres(op, b, max_iter=100, restart=30, rtol=rtol, atol=0.0, preconditioner=O.op_diagonal(np.full(6, 1e3)))
    assert r["converged"]
    true = np.linalg.norm(b - a @ r["x"])
    assert r["residual_norm"] == pytest.approx(1e3 * true, rel=1e-10)
    assert 1e3 * true <= rtol * np.linalg.norm(b)
    # the same solve unpreconditioned stops earlier or at the same step, at
    # a true residual up to 1000x larger
    r0 = O.gmres(op, b, max_iter=100, restart=30, rtol=rtol, atol=0.0)
    assert r0["converged"] and r0["iterations"] <= r["iterations"]


def test_breakdown_threshold_is_absolute():
    a, b = _matrix(scale=1e3)
    r = O.gmres(_op(a), b, max_iter=100, restart=30, rtol=1e-10, atol=0.0)
    # the sixth step counts (h ~ 1e-13 > 10 eps) and completes the space
    assert r["converged"] and r["iterations"] == 6
    sol = np.linalg.solve(a, b)
    assert np.linalg.norm(r["x"] - sol) <= 1e-9 * np.linalg.norm(sol)

    a, b = _matrix(scale=1e-6)
    r = O.gmres(_op(a), b, max_iter=6, restart=30, rtol=1e-14, atol=0.0)
    # the sixth column (h ~ 1e-22 < 10 eps) is dropped: five steps, then one
    # step of a second cycle from x_5
    x5 = _krylov_min(a, np.eye(6), b, np.zeros(6), 5)
    x6 = _krylov_min(a, np.eye(6), b, x5, 1)
    assert r["iterations"] == 6 and not r["converged"]
    assert np.linalg.norm(r["x"] - x6) <= 1e-9 * np.linalg.norm(x6)


def test_a_cycle_that_cannot_advance_is_an_error():
    b = np.array([1.0, -2.0, 0.5, 3.0, 1.5])
    with pytest.raises(ValueError, match="gmres cannot advance"):
        O.gmres(O.op_diagonal(np.full(5, 2.0)), b)  # A r0 = 2 r0: breakdown at step 1
    a, b3 = _matrix(n=3)
    with pytest.raises(ValueError, match="restart = 0 makes no progress"):
        O.gmres(_op(a), b3, restart=0)
    # a zero right-hand side converges before any cycle, whatever the restart
    r = O.gmres(_op(a), np.zeros(3), restart=0)
    assert r["converged"] and r["iterations"] == 0
