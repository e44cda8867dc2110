"""The allocation-free FP64 residual entry point (GPU).

sx_true_rel_residual_noalloc serves callers that cannot allocate device
memory while they run -- a framework whose pool owns all GPU memory, or a
real-time loop that must not stall on an allocation.  It keeps its reduction
scratch in a file-scope device array instead.  This file is collected last so
that a failure here never hides the other tests; it also passes on its own
in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_residual_matches_allocating_entry_point():
    import torch

    import scirs_gb300 as S
    from scirs_gb300 import _lib as L

    ctx = S.Context(0)
    try:
        ip, ix, v = S.generate("varcoef3d", 40, 36, 30, seed=5, param0=1.5)
        n = len(ip) - 1
        a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        b = S.rhs_normal(21, n)
        x = S.rhs_normal(22, n) * 1e-3
        ref = S.true_rel_residual(a, b, x)  # the allocating entry point
        bd = torch.from_numpy(b).cuda()
        xd = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        for _ in range(2):  # two calls in a row share the same scratch
            out = C.c_double()
            S.sparse._check(L.lib.sx_true_rel_residual_noalloc(
                ctx.handle, a.handle, C.c_void_p(bd.data_ptr()), C.c_void_p(xd.data_ptr()), C.byref(out)))
            # residual entries are bit-identical; the norms' summation order differs
            assert abs(out.value - ref) <= 1e-14 * ref, (out.value, ref)
        # a second matrix of another size right after: the counter was cleared
        ip2, ix2, v2 = S.generate("poisson2d", 300, 200)
        n2 = len(ip2) - 1
        a2 = S.csr_from_arrays(ctx, ip2, ix2, v2, (n2, n2))
        b2, x2 = S.rhs_normal(1, n2), S.rhs_normal(2, n2)
        ref2 = S.true_rel_residual(a2, b2, x2)
        bd2 = torch.from_numpy(b2).cuda()  # held: the pointers must stay valid
        xd2 = torch.from_numpy(x2).cuda()
        torch.cuda.synchronize()
        out = C.c_double()
        S.sparse._check(L.lib.sx_true_rel_residual_noalloc(
            ctx.handle, a2.handle, C.c_void_p(bd2.data_ptr()), C.c_void_p(xd2.data_ptr()), C.byref(out)))
        assert abs(out.value - ref2) <= 1e-14 * ref2
        a.close()
        a2.close()
    finally:
        ctx.close()


def test_noalloc_residual_rejects_too_many_rows():
    import torch

    import scirs_gb300 as S
    from scirs_gb300 import _lib as L

    ctx = S.Context(0)
    try:
        n = 16777216 + 1
        a = S.csr_from_arrays(ctx, np.zeros(n + 1, dtype=np.int64), np.zeros(0, dtype=np.int32),
                              np.zeros(0), (n, n))
        # full-size buffers, so that even a launch would stay in bounds
        bd = torch.ones(n, dtype=torch.float64, device="cuda")
        xd = torch.zeros(n, dtype=torch.float64, device="cuda")
        out = C.c_double()
        rc = L.lib.sx_true_rel_residual_noalloc(ctx.handle, a.handle, C.c_void_p(bd.data_ptr()),
                                                C.c_void_p(xd.data_ptr()), C.byref(out))
        assert rc == 9  # SX_ERR_VALUE
        info = L.ErrorInfo()
        L.lib.sx_last_error(C.byref(info))
        assert b"at most 16777216 rows" in info.message
        a.close()
    finally:
        ctx.close()
