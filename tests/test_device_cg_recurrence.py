"""CG in two kernels per iteration (sx_ctx_set_cg_recurrence) against the
oracle (GPU).

With a Jacobi (or no) preconditioner the recurrence variant carries A p as
q = A z + beta q; every other operation keeps the reference loop's roundings
(iterative.rs:95-151).  Its iterates therefore differ from the reference's by
the recurrence's rounding only: the same exit, the iteration count within a
few, and solutions within the tolerance of the solve, on the 2D Poisson 256^2
configuration (FP64) and a 3D variable-coefficient problem (FP64 and FP32).
It takes two kernels per iteration where the reference loop takes three.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _solve(S, ctx, ip, ix, v, b, dtype, recur, rtol, max_iter):
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, v.astype(dtype), (n, n))
    m = S.jacobi(ctx, a)
    ctx.set_cg_recurrence(recur)
    try:
        l0 = ctx.kernel_launches
        r = S.cg(a, b.astype(dtype), max_iter=max_iter, rtol=rtol, atol=0.0, preconditioner=m)
        launches = ctx.kernel_launches - l0
    finally:
        ctx.set_cg_recurrence(False)
        m.close()
        a.close()
    return r, launches


def test_poisson_256_fp64_recurrence_matches_oracle(S):
    ctx = S.Context(0)
    try:
        ip, ix, v = O.generate("poisson2d", 256, 256)
        n = len(ip) - 1
        b = O.rhs_normal(11, n)
        oa = O.op_csr_i32(ip, ix, v, (n, n))
        ro = O.cg(oa, b, max_iter=5000, rtol=1e-10, atol=0.0, preconditioner=O.op_jacobi(oa))
        r3, l3 = _solve(S, ctx, ip, ix, v, b, np.float64, False, 1e-10, 5000)
        r2, l2 = _solve(S, ctx, ip, ix, v, b, np.float64, True, 1e-10, 5000)
        assert ro["converged"] and r2.converged and r3.converged
        assert abs(r2.iterations - ro["iterations"]) <= 4
        scale = np.linalg.norm(ro["x"])
        assert np.linalg.norm(r2.x - ro["x"]) <= 1e-8 * scale
        assert O.true_rel_residual(ip, ix, v, b, r2.x) <= 1.01e-10
        # two kernels per iteration against three (plus a fixed setup)
        assert l2 <= 0.8 * l3
    finally:
        ctx.close()


@pytest.mark.parametrize("dtype,rtol", [(np.float64, 1e-10), (np.float32, 1e-5)])
def test_varcoef3d_recurrence(S, dtype, rtol):
    ctx = S.Context(0)
    try:
        ip, ix, v = O.generate("varcoef3d", 40, 40, 40, seed=3, param0=1.5)
        n = len(ip) - 1
        b = O.rhs_normal(12, n)
        r3, _ = _solve(S, ctx, ip, ix, v, b, dtype, False, rtol, 4000)
        r2, _ = _solve(S, ctx, ip, ix, v, b, dtype, True, rtol, 4000)
        assert r2.converged and r3.converged
        assert abs(r2.iterations - r3.iterations) <= max(4, 0.02 * r3.iterations)
        res = O.true_rel_residual(ip, ix, v.astype(dtype).astype(np.float64), b.astype(dtype).astype(np.float64),
                                  r2.x.astype(np.float64))
        assert res <= (1.5 * rtol if dtype == np.float64 else 20 * rtol)
    finally:
        ctx.close()


def test_recurrence_max_iter_and_zero_rhs(S):
    # the loop's exits: max_iter reached, and b = 0 (the oracle's exit)
    ctx = S.Context(0)
    try:
        ip, ix, v = O.generate("poisson2d", 40, 40)
        n = len(ip) - 1
        b = O.rhs_normal(13, n)
        r, _ = _solve(S, ctx, ip, ix, v, b, np.float64, True, 1e-14, 7)
        ro = O.cg(O.op_csr_i32(ip, ix, v, (n, n)), b, max_iter=7, rtol=1e-14, atol=0.0,
                  preconditioner=O.op_jacobi(O.op_csr_i32(ip, ix, v, (n, n))))
        assert r.iterations == ro["iterations"] == 7 and not r.converged and not ro["converged"]
        assert np.linalg.norm(r.x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
        r0, _ = _solve(S, ctx, ip, ix, v, np.zeros(n), np.float64, True, 1e-8, 100)
        ro0 = O.cg(O.op_csr_i32(ip, ix, v, (n, n)), np.zeros(n), max_iter=100, rtol=1e-8, atol=0.0,
                   preconditioner=O.op_jacobi(O.op_csr_i32(ip, ix, v, (n, n))))
        assert r0.iterations == ro0["iterations"] and r0.converged == ro0["converged"]
        assert np.all(r0.x == 0)
    finally:
        ctx.close()
