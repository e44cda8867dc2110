"""The learned solve with its fallback: the learned factor in the FP32
mixed loop, and plain FP64 Jacobi-PCG from the last iterate when that loop
stops short of the target.  The oracle's FP64 true residual checks both."""
import os

import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_learned_solve_and_jacobi_fallback(ctx):
    import scirs_gb300 as S
    from scirs_gb300 import learned as LR

    pr = LR.sample_problem(7)
    ip, ix, v = S.generate("aniso_q1", 64, 64, param0=pr.eps, param1=pr.theta)
    n = len(ip) - 1
    a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    b = S.rhs_normal(11, n)
    net = LR.load_weights(ctx, os.path.join(REPO, "scirs_gb300", "weights", "aniso_q1.npz"))
    r = LR.solve(net, a64, b, tol=1e-8)
    assert r.converged and r.method == "learned-mixed" and r.fallback_iterations == 0
    assert O.true_rel_residual(ip, ix, v, b, r.x) <= 1.01e-8
    # one short segment: the mixed loop stops unconverged and FP64 Jacobi-PCG
    # finishes from its iterate
    f = LR.solve(net, a64, b, tol=1e-8, max_inner=20, max_outer=1)
    assert f.method == "learned-mixed+jacobi-pcg" and f.inner_iterations <= 20
    assert f.converged and f.fallback_iterations > 0
    assert O.true_rel_residual(ip, ix, v, b, f.x) <= 1.01e-8
    assert abs(f.rel_residual - O.true_rel_residual(ip, ix, v, b, f.x)) <= 1e-12
    net.close()
    a64.close()
