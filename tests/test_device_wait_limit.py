"""Bounded device waits run out and report, without a GPU fault (GPU).

The triangular factorisations and sweeps (IC(0), ILU(0), SSOR) order their
rows by flag waits, each bounded by the context's wait limit (2 s by
default).  A wait that runs out raises an abort flag that ends every other
wait of the launch, and the call returns SX_ERR_DEVICE_TIMEOUT; the context
stays usable.  Here the limit is made short so that waits do run out: first
on a flag that nothing sets, then inside a multi-level IC(0) apply.  With
the default limit restored, the same context and operator give the
oracle's bits again and a preconditioned solve converges.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu

SX_ERR_DEVICE_TIMEOUT = 101


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def test_wait_on_unset_flag_gives_up_at_the_limit(S):
    from scirs_gb300 import _lib as L

    ctx = S.Context(0)
    try:
        limit = 1_000_000  # 1 ms
        S.sparse._check(L.lib.sx_ctx_set_wait_limit(ctx.handle, limit))
        waited = C.c_uint64()
        rc = L.lib.sx_wait_selftest(ctx.handle, C.byref(waited))
        assert rc == SX_ERR_DEVICE_TIMEOUT
        assert limit <= waited.value < 1000 * limit
        info = L.ErrorInfo()
        L.lib.sx_last_error(C.byref(info))
        assert b"Device timeout" in info.message
        # the context keeps working: a device SpMV right after
        ip, ix, v = S.generate("poisson2d", 30, 30)
        n = len(ip) - 1
        a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        x = S.rhs_normal(1, n)
        assert np.array_equal(a.matvec(x), O.spmv_i32(ip, ix, v, x))
        a.close()
    finally:
        ctx.close()


def test_ic0_apply_wait_limit_then_default(S):
    from scirs_gb300 import _lib as L

    ctx = S.Context(0)
    try:
        # 2D Q1 256^2: 768 dependency levels in each triangular solve
        ip, ix, v = S.generate("aniso_q1", 256, 256, param0=30.0, param1=0.4)
        n = len(ip) - 1
        a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        m = S.ic0(ctx, a)  # the reference's factorisation, with the default limit
        x = S.rhs_normal(3, n)
        y_ok = m.matvec(x)
        # a 2-microsecond limit: the solves' waits on earlier levels run out
        S.sparse._check(L.lib.sx_ctx_set_wait_limit(ctx.handle, 2000))
        with pytest.raises(S.SparseError) as e:
            m.matvec(x)
        assert e.value.variant == "DeviceTimeout"
        # the default limit again (0): the same operator, the same bits
        S.sparse._check(L.lib.sx_ctx_set_wait_limit(ctx.handle, 0))
        y = m.matvec(x)
        assert np.array_equal(y.view(np.uint8), y_ok.view(np.uint8))
        oa = O.op_csr_i32(ip, ix, v, (n, n))
        assert np.array_equal(y.view(np.uint8), O.op_ic0(oa, fast=True).matvec(x).view(np.uint8))
        b = S.rhs_normal(4, n)
        r = S.cg(a, b, max_iter=2000, rtol=1e-8, atol=0.0, preconditioner=m)
        assert r.converged
        assert O.true_rel_residual(ip, ix, v, b, r.x) <= 1.01e-8
        m.close()
        a.close()
    finally:
        ctx.close()
