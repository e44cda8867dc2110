"""The windowed SpMV: window, warp and run-over boundaries vs the oracle.

The nonzeros stream through per-warp windows; rows that cross a window or
a warp's range carry a partial sum.  These matrices put long rows, empty
rows and one-entry rows across those boundaries.  Bars: exact mode is
bit-identical to the oracle (and to the other kernels, SX_WIN=0); the FP64
fused-multiply-add mode stays within a few ulp of sum_k |a_k x_k|.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _from_lengths(rng, lengths, ncols):
    lengths = np.asarray(lengths, dtype=np.int64)
    ip = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    rows = np.repeat(np.arange(len(lengths)), lengths)
    ix = rng.integers(0, ncols, ip[-1])
    ix = ix[np.lexsort((ix, rows))].astype(np.int32)  # sorted within each row
    v = rng.uniform(-1.0, 1.0, ip[-1])
    return ip, ix, v


def _cases(rng):
    yield "one_huge_row", [3, 70000, 2, 0, 0, 7]
    yield "empties_everywhere", [0, 0, 5, 0, 0, 0, 300, 0, 1, 0, 0] * 500
    yield "empty_tail", [10] * 600 + [0] * 5000
    yield "leading_empty", [0] * 2000 + [256] * 100 + [0] * 3
    yield "exact_units", [256] * 400
    yield "ones", [1] * 300000
    yield "long_rows_across_warps", list(rng.integers(3000, 4097, 300))
    yield "powerlaw", list(np.minimum(4096, (rng.pareto(1.2, 20000) + 1).astype(int)))
    yield "ragged", list(rng.integers(0, 40, 50000))
    yield "single", [1]


def _ctx_with(S, env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return S.Context(0)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


@pytest.mark.parametrize("shape", ["0", "1", "2"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_window_boundaries_bit_exact(S, dtype, shape):
    # SX_WIN=2: the windowed kernel for every matrix, each window shape
    c = _ctx_with(S, {"SX_WIN": "2", "SX_WIN_SHAPE": shape})
    rng = np.random.default_rng(17)
    for name, lengths in _cases(rng):
        ncols = 8000
        ip, ix, v = _from_lengths(rng, lengths, ncols)
        n = len(ip) - 1
        vals = v.astype(dtype)
        a = S.csr_from_arrays(c, ip, ix, vals, (n, ncols))
        x = rng.standard_normal(ncols).astype(dtype)
        y = a.matvec(x)
        yr = O.spmv_i32(ip, ix, vals, x)
        assert np.array_equal(y.view(np.uint8), yr.view(np.uint8)), name
        a.close()
    c.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_sliced_bit_exact(S, ctx, dtype):
    # the default for long-row matrices: rows ordered by length in slices of
    # 32 (big slices summed by one lane each from products staged by the
    # block, mid slices in registers, short slices four per warp); rows
    # longer than the sort's 4096 cap, empty rows, one-entry rows
    rng = np.random.default_rng(23)
    seen = 0
    for name, lengths in _cases(rng):
        ncols = 8000
        ip, ix, v = _from_lengths(rng, lengths, ncols)
        n = len(ip) - 1
        vals = v.astype(dtype)
        a = S.csr_from_arrays(ctx, ip, ix, vals, (n, ncols))
        seen += S.spmv_kernel(a) == "spmv_sliced_kernel"
        x = rng.standard_normal(ncols).astype(dtype)
        y = a.matvec(x)
        assert np.array_equal(y.view(np.uint8), O.spmv_i32(ip, ix, vals, x).view(np.uint8)), name
        # x[0] = inf: rows holding column 0 become +-inf (NaN where column 0
        # repeats with both signs) like the reference's; the padding (column
        # 0, value 0) must never enter a sum.  A NaN's sign bit is the
        # platform's choice (IEEE 754 leaves it open), so NaNs compare by place.
        x[0] = np.inf
        y = a.matvec(x)
        yr = O.spmv_i32(ip, ix, vals, x)
        nan = np.isnan(yr)
        assert np.array_equal(np.isnan(y), nan), name
        assert np.array_equal(y[~nan].view(np.uint8), yr[~nan].view(np.uint8)), name
        a.close()
    assert seen >= 3


def test_windowed_kernel_matches_row_kernel(S):
    # the same products and sums with and without the windowed kernel
    rng = np.random.default_rng(3)
    ip, ix, v = S.generate("powerlaw", 200000, 1, 1, seed=4, param0=16.0, param1=4096.0)
    n = len(ip) - 1
    x = rng.standard_normal(n)
    out = {}
    for mode in ("2", "0"):
        c = _ctx_with(S, {"SX_WIN": mode})
        a = S.csr_from_arrays(c, ip, ix, v, (n, n))
        out[mode] = a.matvec(x)
        a.close()
        c.close()
    assert np.array_equal(out["0"].view(np.uint8), out["2"].view(np.uint8))


@pytest.mark.parametrize("env", [{"SX_WIN": "0", "SX_DIA": "0"}, {"SX_WIN": "2", "SX_DIA": "0"}, {},
                                 {"SX_BIN": "0"}])
@pytest.mark.parametrize("kind,dims", [("laplace3d", (64, 64, 64)), ("powerlaw", (300000, 1, 1))])
def test_fp64_fma_mode_within_ulps(S, kind, dims, env):
    # the CSR kernels (row-wise, windowed) and, for the stencil, the diagonal layout
    ctx = _ctx_with(S, env)
    import torch

    from scirs_gb300 import _lib as L

    p0, p1 = (16.0, 4096.0) if kind == "powerlaw" else (0.0, 0.0)
    ip, ix, v = S.generate(kind, *dims, seed=2, param0=p0, param1=p1)
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    x = np.random.default_rng(8).standard_normal(n)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, a.handle, C.c_void_p(xd.data_ptr()),
                                     C.c_void_p(yd.data_ptr()), 0))
    ctx.synchronize()
    y = yd.cpu().numpy()
    yr = O.spmv_i32(ip, ix, v, x)
    rows = np.repeat(np.arange(n), np.diff(ip))
    mag = np.bincount(rows, weights=np.abs(v * x[ix]), minlength=n)
    lens = np.diff(ip).astype(np.float64)
    # sequential summation error bound: (len + 1) * eps * sum |a x|
    bound = (lens + 1.0) * np.finfo(np.float64).eps * mag
    assert np.all(np.abs(y - yr) <= bound + 1e-300)
    # fused multiply-adds: not the exact mode's bits on these values
    assert not np.array_equal(y, yr)
    a.close()
    ctx.close()


def test_full_size_laplacian_fp32_bit_exact(S, ctx):
    ip, ix, v = S.generate("laplace3d", 128, 128, 128)
    n = len(ip) - 1
    vals = v.astype(np.float32)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    x = S.rhs_normal(5, n).astype(np.float32)
    y = a.matvec(x)
    yr = O.spmv_i32(ip, ix, vals, x)
    assert np.array_equal(y.view(np.uint8), yr.view(np.uint8))
    a.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind,dims,p0,p1", [
    ("laplace3d", (48, 40, 36), 0.0, 0.0),
    ("aniso_q1", (200, 150, 1), 300.0, 0.5),
    ("varcoef3d", (30, 30, 30), 1.5, 0.0),
])
def test_compressed_columns_bit_exact(S, dtype, kind, dims, p0, p1):
    # the register-pipelined SpMV with the int32 columns, with the 16-bit
    # column offsets (stencil spans), and the register-only short-row
    # kernel: all the oracle's bits
    ip, ix, v = S.generate(kind, *dims, seed=6, param0=p0, param1=p1)
    n = len(ip) - 1
    vals = v.astype(dtype)
    x = np.random.default_rng(2).standard_normal(n).astype(dtype)
    yr = O.spmv_i32(ip, ix, vals, x)
    for env in ({}, {"SX_DIA_ND6": "0"}, {"SX_DIA": "0"}, {"SX_DIA": "0", "SX_SHORT": "2"},
                {"SX_DIA": "0", "SX_SHORT": "0", "SX_COL16": "1"}):
        c = _ctx_with(S, env)
        a = S.csr_from_arrays(c, ip, ix, vals, (n, n))
        y = a.matvec(x)
        assert np.array_equal(y.view(np.uint8), yr.view(np.uint8)), env
        a.close()
        c.close()


def test_compressed_columns_wide_rows_keep_int32(S, ctx):
    # a chunk spanning more than 65,535 columns: no compressed copy, same bits
    rng = np.random.default_rng(9)
    n, ncols = 3000, 200000
    lengths = rng.integers(1, 9, n)
    ip = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    rows = np.repeat(np.arange(n), lengths)
    ix = rng.integers(0, ncols, ip[-1])
    ix = ix[np.lexsort((ix, rows))].astype(np.int32)
    v = rng.uniform(-1, 1, ip[-1])
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, ncols))
    x = rng.standard_normal(ncols)
    assert np.array_equal(a.matvec(x).view(np.uint8), O.spmv_i32(ip, ix, v, x).view(np.uint8))
    a.close()



def test_kernel_choice_names(S, ctx):
    # the dispatch: the diagonal layout for stencils; without it (SX_DIA=0)
    # short rows in registers for FP64 with FMA and the register pipeline for
    # FP32 and exact FP64; windows for long rows
    ip, ix, v = S.generate("laplace3d", 20, 20, 20)
    n = len(ip) - 1
    a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    a32 = a64.astype(np.float32)
    # default (SX_DIA=1): the diagonal layout for FP64 and FP32 (7 diagonals
    # in bands 1+1+3+1+1: the three adjacent ones share one x window)
    assert S.spmv_kernel(a32) == "spmv_dia_kernel<ND=7, bands 1+1+3+1+1>"
    assert S.spmv_kernel(a64, exact=False) == "spmv_dia_kernel<ND=7, bands 1+1+3+1+1>"
    assert S.spmv_kernel(a64, exact=True) == "spmv_dia_kernel<ND=7, bands 1+1+3+1+1>"
    cb = _ctx_with(S, {"SX_DIA_BAND": "0"})
    nb32 = S.csr_from_arrays(cb, ip, ix, v.astype(np.float32), (n, n))
    assert S.spmv_kernel(nb32) == "spmv_dia_kernel<ND=7>"
    nb32.close()
    cb.close()
    # five diagonals (the 2D 5-point stencil): the exact-count kernel; the
    # generic one with SX_DIA_ND6=0
    ip5, ix5, v5 = S.generate("poisson2d", 40, 40)
    f32 = S.csr_from_arrays(ctx, ip5, ix5, v5.astype(np.float32), (1600, 1600))
    assert S.spmv_kernel(f32) == "spmv_dia_kernel<ND=5, bands 1+3+1>"
    c2 = _ctx_with(S, {"SX_DIA_ND6": "0"})
    d32 = S.csr_from_arrays(c2, ip5, ix5, v5.astype(np.float32), (1600, 1600))
    assert S.spmv_kernel(d32) == "spmv_dia_kernel<ND=16>"
    d32.close()
    f32.close()
    c2.close()
    c = _ctx_with(S, {"SX_DIA": "0"})
    b64 = S.csr_from_arrays(c, ip, ix, v, (n, n))
    b32 = b64.astype(np.float32)
    assert S.spmv_kernel(b32) == "spmv_pipe_kernel<ITEMS=8>"
    assert S.spmv_kernel(b64, exact=False) == "spmv_short_kernel<K=8>"
    assert S.spmv_kernel(b64, exact=True) == "spmv_pipe_kernel<ITEMS=8>"
    ip, ix, v = S.generate("powerlaw", 50000, 1, 1, seed=2, param0=16.0, param1=4096.0)
    n = len(ip) - 1
    p = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    assert S.spmv_kernel(p) == "spmv_sliced_kernel"
    assert S.spmv_kernel(p, exact=False) == "spmv_sliced_kernel<FMA>"
    p32 = p.astype(np.float32)
    assert S.spmv_kernel(p32) == "spmv_sliced_kernel"
    p32.close()
    cw = _ctx_with(S, {"SX_BIN": "0"})
    pw = S.csr_from_arrays(cw, ip, ix, v, (n, n))
    assert S.spmv_kernel(pw) == "spmv_win_kernel"
    for op in (a32, a64, b32, b64, p, pw):
        op.close()
    c.close()
    cw.close()


def _diag_cases(rng):
    # (name, indptr, indices, values, expect the diagonal layout)
    n = 4000
    offs = [-37, -1, 0, 1, 5, 300]
    rows, cols = [], []
    for i in range(n):
        for o in offs:
            j = i + o
            if 0 <= j < n and rng.uniform() < 0.9:  # ragged: absent entries inside the band
                rows.append(i)
                cols.append(j)
    rows, cols = np.asarray(rows), np.asarray(cols)
    ip = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int64)
    v = rng.uniform(-1, 1, len(cols))
    yield "banded_ragged", ip, cols.astype(np.int32), v, True
    # the same rows with one pair of columns swapped: not strictly increasing
    c2 = cols.copy()
    k = int(ip[100])
    c2[k], c2[k + 1] = c2[k + 1], c2[k]
    yield "unsorted_row", ip, c2.astype(np.int32), v, False
    # a duplicate entry
    c3 = cols.copy()
    c3[k + 1] = c3[k]
    yield "duplicate", ip, c3.astype(np.int32), v, False
    # 17 diagonals
    offs17 = list(range(-8, 9))
    rows = np.repeat(np.arange(n), len(offs17))
    cols = (rows + np.tile(offs17, n))
    keep = (cols >= 0) & (cols < n)
    rows, cols = rows[keep], cols[keep]
    ip = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int64)
    yield "seventeen_diagonals", ip, cols.astype(np.int32), rng.uniform(-1, 1, len(cols)), False


@pytest.mark.parametrize("env", [{}, {"SX_DIA_ND6": "0"}])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_diagonal_layout_bit_exact(S, dtype, env):
    rng = np.random.default_rng(12)
    ctx = _ctx_with(S, env)
    for name, ip, ix, v, expect in _diag_cases(rng):
        n = len(ip) - 1
        vals = v.astype(dtype)
        a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
        assert S.spmv_kernel(a).startswith("spmv_dia") == expect, name
        x = rng.standard_normal(n).astype(dtype)
        # one infinite x: the rows that store its column give +-inf; a padded
        # (absent) entry multiplied into it would give NaN
        x[n // 2] = np.inf
        y = a.matvec(x)
        assert np.array_equal(y.view(np.uint8), O.spmv_i32(ip, ix, vals, x).view(np.uint8)), name
        a.close()
    ctx.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_diagonal_layout_unaligned_vectors(S, dtype):
    # device vectors that do not start on 16 bytes (an odd element offset)
    # take the CSR kernels: the same bits, no misaligned vector access
    import torch

    from scirs_gb300 import _lib as L

    ctx = S.Context(0)
    ip, ix, v = S.generate("poisson2d", 33, 31)
    n = len(ip) - 1
    vals = v.astype(dtype)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    assert S.spmv_kernel(a).startswith("spmv_dia")
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    x = np.random.default_rng(3).standard_normal(n).astype(dtype)
    xb = torch.zeros(n + 1, dtype=tdt, device="cuda")
    yb = torch.zeros(n + 1, dtype=tdt, device="cuda")
    xb[1:] = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    for flags in (1, 0) if dtype == np.float64 else (1,):
        S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, a.handle, C.c_void_p(xb.data_ptr() + xb.element_size()),
                                         C.c_void_p(yb.data_ptr() + yb.element_size()), flags))
        ctx.synchronize()
        y = yb[1:].cpu().numpy()
        yr = O.spmv_i32(ip, ix, vals, x)
        if flags == 1:
            assert np.array_equal(y.view(np.uint8), yr.view(np.uint8))
        else:
            assert np.allclose(y, yr, rtol=1e-14, atol=1e-14)
    a.close()
    ctx.close()


def _tri(ip, ix, v, lower):
    # the lower (or upper) triangle of a CSR matrix, diagonal included
    rows = np.repeat(np.arange(len(ip) - 1), np.diff(ip))
    keep = ix <= rows if lower else ix >= rows
    cnt = np.bincount(rows[keep], minlength=len(ip) - 1)
    ptr = np.zeros(len(ip), np.int64)
    ptr[1:] = np.cumsum(cnt)
    return ptr, ix[keep], v[keep]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_band_kernels_bit_exact(S, ctx, dtype):
    # every band shape the exact-count kernels specialise (Q1: 3+3+3; 3D
    # 7-point: 1+1+3+1+1; 2D 5-point: 1+3+1; the learned factors' lower and
    # upper Q1 triangles: 3+2 and 2+3) on grids small enough that many rows
    # are boundary rows: the oracle's bits, with and without bands, and with
    # an infinite x entry
    cases = [
        ("aniso_q1", (37, 29), dict(param0=30.0, param1=0.4), "bands 3+3+3", None),
        ("laplace3d", (11, 9, 13), {}, "bands 1+1+3+1+1", None),
        ("poisson2d", (33, 21), {}, "bands 1+3+1", None),
        ("aniso_q1", (41, 23), dict(param0=8.0, param1=1.1), "bands 3+2", True),
        ("aniso_q1", (26, 31), dict(param0=8.0, param1=1.1), "bands 2+3", False),
        ("aniso_q1", (3, 2), dict(param0=2.0, param1=0.3), "bands 3+3+3", None),
    ]
    cb = _ctx_with(S, {"SX_DIA_BAND": "0"})
    rng = np.random.default_rng(41)
    try:
        for kind, dims, kw, shape, lower in cases:
            ip, ix, v = S.generate(kind, *dims, **kw)
            if lower is not None:
                ip, ix, v = _tri(ip, ix, v, lower)
            n = len(ip) - 1
            vals = v.astype(dtype)
            a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
            b = S.csr_from_arrays(cb, ip, ix, vals, (n, n))
            if n >= 64:
                assert shape in S.spmv_kernel(a), (kind, dims, S.spmv_kernel(a))
            for trial in range(2):
                x = rng.standard_normal(n).astype(dtype)
                if trial:
                    x[n // 2] = np.inf
                y = a.matvec(x)
                yr = O.spmv_i32(ip, ix, vals, x)
                nan = np.isnan(yr)
                assert np.array_equal(np.isnan(y), nan), (kind, dims)
                assert np.array_equal(y[~nan].view(np.uint8), yr[~nan].view(np.uint8)), (kind, dims)
                yb = b.matvec(x)
                assert np.array_equal(np.isnan(yb), nan), (kind, dims)
                assert np.array_equal(yb[~nan].view(np.uint8), yr[~nan].view(np.uint8)), (kind, dims)
            a.close()
            b.close()
    finally:
        cb.close()


def test_programmatic_launch_same_bits(S):
    # SpMVs launched with programmatic dependent launch (the default) and
    # without (SX_PDL=0): the same products and solver runs, bit for bit
    ip, ix, v = S.generate("aniso_q1", 96, 80, param0=40.0, param1=0.7)
    n = len(ip) - 1
    b = np.random.default_rng(5).standard_normal(n)
    out = {}
    for mode in ("1", "0"):
        c = _ctx_with(S, {"SX_PDL": mode})
        a = S.csr_from_arrays(c, ip, ix, v, (n, n))
        a32 = a.astype(np.float32)
        m = S.jacobi(c, a)
        m32 = S.jacobi(c, a32)
        r = S.cg(a, b, max_iter=5000, rtol=1e-10, atol=0.0, preconditioner=m)
        rm = S.cg_mixed(a, b, tol=1e-9, preconditioner=m32, a32=a32)
        out[mode] = (a32.matvec(b.astype(np.float32)), r.iterations, r.x, rm.inner_iterations, rm.x)
        for op in (m, m32, a32, a):
            op.close()
        c.close()
    y1, it1, x1, im1, xm1 = out["1"]
    y0, it0, x0, im0, xm0 = out["0"]
    assert np.array_equal(y1.view(np.uint8), y0.view(np.uint8))
    assert it1 == it0 and np.array_equal(x1.view(np.uint8), x0.view(np.uint8))
    assert im1 == im0 and np.array_equal(xm1.view(np.uint8), xm0.view(np.uint8))
