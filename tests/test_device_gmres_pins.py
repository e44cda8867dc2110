"""gmres known answers on the device (GPU).

The device gmres (sx_gmres) against the same mathematical pins as the
oracle's restatement (tests/test_oracle_gmres.py): each cycle minimises the
residual over its Krylov space, restarted cycles chain those minimisations,
the breakdown test is absolute (10 eps), and a cycle that cannot advance
ends with an error where the reference's loop (iterative.rs:697-808)
repeats it forever.
"""
import numpy as np
import pytest

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


def _matrix(scale=1.0, n=6, seed=3):
    rng = np.random.default_rng(seed)
    a = (4.0 * np.eye(n) + 0.6 * rng.standard_normal((n, n))) * scale
    b = rng.standard_normal(n)
    return a, b


def _csr(S, ctx, a):
    n = a.shape[0]
    ip = np.arange(0, n * n + 1, n, dtype=np.int64)
    ix = np.tile(np.arange(n, dtype=np.int32), n)
    return S.csr_from_arrays(ctx, ip, ix, a.ravel().copy(), (n, n))


def _krylov_min(a, b, x0, k):
    r0 = b - a @ x0
    q = [r0 / np.linalg.norm(r0)]
    for _ in range(k - 1):
        w = a @ q[-1]
        for _ in range(2):
            for v in q:
                w = w - (v @ w) * v
        q.append(w / np.linalg.norm(w))
    basis = np.stack(q, 1)
    return x0 + basis @ np.linalg.lstsq(a @ basis, r0, rcond=None)[0]


@pytest.mark.parametrize("k", [1, 3, 5])
def test_cycle_minimises_over_the_krylov_space(S, ctx, k):
    a, b = _matrix()
    op = _csr(S, ctx, a)
    r = S.gmres(op, b, max_iter=k, restart=30, rtol=1e-14, atol=0.0)
    ref = _krylov_min(a, b, np.zeros(6), k)
    assert r.iterations == k and not r.converged
    assert np.linalg.norm(r.x - ref) <= 1e-10 * np.linalg.norm(ref)
    op.close()


def test_restarted_cycles_chain_minimisations(S, ctx):
    a, b = _matrix()
    op = _csr(S, ctx, a)
    r = S.gmres(op, b, max_iter=5, restart=2, rtol=1e-14, atol=0.0)
    x = np.zeros(6)
    for k in (2, 2, 1):
        x = _krylov_min(a, b, x, k)
    assert r.iterations == 5
    assert np.linalg.norm(r.x - x) <= 1e-10 * np.linalg.norm(x)
    op.close()


def test_breakdown_threshold_is_absolute(S, ctx):
    a, b = _matrix(scale=1e3)
    op = _csr(S, ctx, a)
    r = S.gmres(op, b, max_iter=100, restart=30, rtol=1e-10, atol=0.0)
    assert r.converged and r.iterations == 6
    op.close()
    a, b = _matrix(scale=1e-6)
    op = _csr(S, ctx, a)
    r = S.gmres(op, b, max_iter=6, restart=30, rtol=1e-14, atol=0.0)
    x6 = _krylov_min(a, b, _krylov_min(a, b, np.zeros(6), 5), 1)
    assert r.iterations == 6 and not r.converged
    assert np.linalg.norm(r.x - x6) <= 1e-9 * np.linalg.norm(x6)
    op.close()


def test_a_cycle_that_cannot_advance_is_an_error(S, ctx):
    n = 5
    op = _csr(S, ctx, 2.0 * np.eye(n))
    with pytest.raises(S.SparseError) as e:
        S.gmres(op, np.array([1.0, -2.0, 0.5, 3.0, 1.5]))
    assert e.value.variant == "ComputationError"
    assert "gmres cannot advance" in str(e.value)
    # the context stays usable: a regular solve right after
    a, b = _matrix()
    op2 = _csr(S, ctx, a)
    r = S.gmres(op2, b, rtol=1e-10, atol=0.0)
    assert r.converged
    op.close()
    op2.close()
