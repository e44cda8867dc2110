"""ILU(0) and SSOR on the device vs the oracle (preconditioners.rs:94-399).

Factorisation and apply are bit-identical with the oracle's restatement of
the reference's loops, also for unsorted rows with duplicate entries, where
the reference's column search stops at the first larger column; the errors
name the same first failing row; the preconditioned solvers match the
oracle's iteration counts.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


def random_csr(rng, n, extra=4, unsorted=False, dups=False):
    """Diagonally dominant CSR arrays (int64 indptr, int32 indices)."""
    rows = []
    for i in range(n):
        cols = list(rng.choice(n, size=min(extra, n), replace=False))
        if i not in cols:
            cols.append(i)
        if dups and rng.uniform() < 0.3:
            cols.append(cols[rng.integers(0, len(cols))])
        cols = list(rng.permutation(cols)) if unsorted else sorted(cols)
        vals = [rng.uniform(-1.0, 1.0) for _ in cols]
        off = sum(abs(v) for c, v in zip(cols, vals) if c != i)
        for t, c in enumerate(cols):
            if c == i:
                vals[t] = off + 1.0 + rng.uniform()
        rows.append((cols, vals))
    ip = np.concatenate([[0], np.cumsum([len(c) for c, _ in rows])]).astype(np.int64)
    ix = np.concatenate([np.asarray(c, dtype=np.int32) for c, _ in rows])
    v = np.concatenate([np.asarray(vv) for _, vv in rows])
    return ip, ix, v


def _cases(S):
    rng = np.random.default_rng(3)
    yield "random_sorted", random_csr(rng, 3000)
    yield "random_unsorted_dups", random_csr(rng, 3000, unsorted=True, dups=True)
    ip, ix, v = S.generate("poisson2d", 64, 64)
    yield "poisson64", (ip, ix, v)
    from scirs_gb300 import learned as LR

    pr = LR.sample_problem(7)
    ip, ix, v = S.generate("aniso_q1", 40, 40, param0=pr.eps, param1=pr.theta)
    yield "aniso_q1_40", (ip, ix, v)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_apply_bit_exact(S, ctx, dt):
    for name, (ip, ix, v) in _cases(S):
        n = len(ip) - 1
        v = v.astype(dt)
        a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        oa = O.op_csr_i32(ip, ix, v, (n, n), f64=dt == np.float64)
        x = np.random.default_rng(11).standard_normal(n).astype(dt)
        m = S.ilu0(ctx, a)
        om = O.op_ilu0(oa)
        assert np.array_equal(_bits(m.matvec(x)), _bits(om.matvec(x))), (name, "ilu0")
        for omega in (1.0, 0.7, 1.6):
            s = S.ssor(ctx, a, omega)
            os_ = O.op_ssor(oa, omega)
            assert np.array_equal(_bits(s.matvec(x)), _bits(os_.matvec(x))), (name, "ssor", omega)
        assert not m.has_adjoint and not s.has_adjoint
        with pytest.raises(S.SparseError, match="adjoint not implemented for this operator"):
            m.rmatvec(x)


def test_errors_match_oracle(S, ctx):
    a = S.csr_matrix(ctx, [1.0, 1.0], [0, 1], [0, 1], (2, 2))
    for om in (0.0, 2.0, -0.5):
        with pytest.raises(S.SparseError, match=r"Value error: Relaxation parameter omega must be in \(0, 2\)"):
            S.ssor(ctx, a, om)
    # row 3 lacks its diagonal; row 1 has a zero pivot after elimination
    rows = [0, 0, 1, 1, 2, 3, 3]
    cols = [0, 1, 0, 1, 2, 0, 2]
    data = [1.0, 1.0, 1.0, 1.0, 5.0, 1.0, 1.0]
    a = S.csr_matrix(ctx, data, rows, cols, (4, 4))
    with pytest.raises(S.SparseError, match="Value error: Zero pivot at position 1"):
        S.ilu0(ctx, a)
    rows2 = [0, 1, 2, 3]
    cols2 = [0, 1, 2, 1]
    a2 = S.csr_matrix(ctx, [1.0, 2.0, 3.0, 4.0], rows2, cols2, (4, 4))
    with pytest.raises(S.SparseError, match="Value error: Missing diagonal element at row 3"):
        S.ilu0(ctx, a2)
    with pytest.raises(S.SparseError, match="Value error: Zero diagonal element at position 3"):
        S.ssor(ctx, a2, 1.0)
    for rr, cc, dd in ((rows, cols, data), (rows2, cols2, [1.0, 2.0, 3.0, 4.0])):
        ip = np.zeros(5, dtype=np.uint64)
        order = np.lexsort((cc, rr))
        np.add.at(ip, np.asarray(rr) + 1, 1)
        ip = np.cumsum(ip).astype(np.uint64)
        oa = O.op_csr(ip, np.asarray(cc, dtype=np.uint64)[order], np.asarray(dd)[order], (4, 4))
        with pytest.raises(ValueError):
            O.op_ilu0(oa)
    rect = S.csr_matrix(ctx, [1.0], [0], [0], (2, 3))
    with pytest.raises(S.SparseError, match="Dimension mismatch: expected 2, found 3"):
        S.ilu0(ctx, rect)


def test_preconditioned_solvers_match_oracle(S, ctx):
    # a 2D 5-point matrix with non-symmetric values and a diagonal shift
    ip, ix, v = S.generate("poisson2d", 32, 32)
    n = len(ip) - 1
    rng = np.random.default_rng(5)
    v = v * (1.0 + 0.1 * rng.standard_normal(len(v)))
    rows = np.repeat(np.arange(n), np.diff(ip))
    v[ix == rows] += 0.5
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    b = S.rhs_normal(4, n)
    for mk, omk in ((lambda: S.ilu0(ctx, a), lambda: O.op_ilu0(oa)),
                    (lambda: S.ssor(ctx, a, 1.3), lambda: O.op_ssor(oa, 1.3))):
        m, om = mk(), omk()
        d = S.gmres(a, b, rtol=1e-8, atol=0.0, preconditioner=m)
        o = O.gmres(oa, b, rtol=1e-8, atol=0.0, preconditioner=om)
        assert d.converged and o["converged"]
        assert abs(d.iterations - o["iterations"]) <= max(2, 0.05 * o["iterations"])
        plain = S.gmres(a, b, rtol=1e-8, atol=0.0)
        assert d.iterations < plain.iterations
        # bicgstab runs its loop in a CUDA graph with the sweeps inside
        d = S.bicgstab(a, b, rtol=1e-8, atol=0.0, right_preconditioner=m)
        o = O.bicgstab(oa, b, rtol=1e-8, atol=0.0, right=om)
        assert d.converged and o["converged"]
        assert abs(d.iterations - o["iterations"]) <= max(2, 0.1 * o["iterations"])
        assert np.linalg.norm(d.x - o["x"]) <= 1e-6 * np.linalg.norm(o["x"])
