"""The oracle's restatement of the mixed-precision loops (no reference
counterpart): both meet the FP64 true-residual target on CPU."""
import numpy as np

from oracle import oracle_ffi as O


def test_mixed_precision_oracles_reach_fp64_tolerance():
    # the two refinement loops of the mixed-precision restatement (no
    # reference counterpart): both meet the FP64 true-residual target, and
    # residual replacement keeps the Krylov progress (fewer FP32 iterations)
    import scirs_gb300 as S  # seeded generators (host code only)

    ip, ix, v = S.generate("varcoef3d", 20, 18, 16, seed=2, param0=1.5)
    n = len(ip) - 1
    b = S.rhs_normal(4, n)
    r1 = O.cg_mixed_ir(ip, ix, v, b, tol=1e-10, inner_rtol=1e-4)
    r2 = O.cg_mixed_replace(ip, ix, v, b, tol=1e-10)
    assert r1["converged"] and r2["converged"]
    for r in (r1, r2):
        assert O.true_rel_residual(ip, ix, v, b, r["x"]) <= 1e-10
    assert r2["inner"] < r1["inner"]
    assert np.linalg.norm(r1["x"] - r2["x"]) / np.linalg.norm(r1["x"]) < 1e-7
