"""The device block cache (GPU).

Freed device arrays are held for reuse instead of going back through
cudaFree; a held block is handed out again only after the work queued on
the context streams at its free has completed.  Repeated solves that free
and reallocate every array must give identical results, and
sx_mem_cache_trim must return every held block.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def test_reused_blocks_give_identical_solves(S):
    ctx = S.Context(0)
    try:
        ip, ix, v = O.generate("poisson2d", 160, 150)
        n = len(ip) - 1
        b = O.rhs_normal(3, n)
        runs = []
        for _ in range(3):
            a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
            m = S.jacobi(ctx, a)
            runs.append(S.cg(a, b, max_iter=3000, rtol=1e-10, atol=0.0, preconditioner=m))
            y = a.matvec(b)
            m.close()
            a.close()
            assert S.mem_cache_bytes() > 0
            assert np.array_equal(y, O.spmv_i32(ip, ix, v, b))
        for r in runs[1:]:
            assert r.iterations == runs[0].iterations
            assert np.array_equal(r.x, runs[0].x)
        S.mem_cache_trim()
        assert S.mem_cache_bytes() == 0
    finally:
        ctx.close()


def test_blocks_freed_on_one_context_serve_another(S):
    # a block freed on one context's stream and reused by a second context:
    # the second context's results do not depend on where its arrays came from
    ip, ix, v = O.generate("varcoef3d", 30, 28, 26, seed=2, param0=1.0)
    n = len(ip) - 1
    b = O.rhs_normal(4, n)
    c1 = S.Context(0)
    c2 = S.Context(0)
    try:
        a1 = S.csr_from_arrays(c1, ip, ix, v, (n, n))
        r1 = S.cg(a1, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.jacobi(c1, a1))
        a1.close()
        a2 = S.csr_from_arrays(c2, ip, ix, v, (n, n))
        r2 = S.cg(a2, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=S.jacobi(c2, a2))
        a2.close()
        assert r1.iterations == r2.iterations
        assert np.array_equal(r1.x, r2.x)
    finally:
        c1.close()
        c2.close()
