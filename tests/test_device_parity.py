"""Device library vs CPU oracle on seeded inputs.

Bars: CSR construction and transpose bit-exact; SpMV bit-exact (the device
sums each row in storage order with separately rounded products, like the
reference); solvers within the stated tolerances.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def oracle_matrix_new(rows, cols, data, shape):
    f64 = data.dtype == np.float64
    nnz = len(data)
    ip = np.empty(shape[0] + 1, dtype=np.uint64)
    ix = np.empty(nnz, dtype=np.uint64)
    d = np.empty(nnz, dtype=data.dtype)
    e = O.Err()
    f = O.lib().or_csr_matrix_new_f64 if f64 else O.lib().or_csr_matrix_new_f32
    rc = f(O.p(data), O.p(rows), O.p(cols), nnz, shape[0], shape[1], O.p(ip), O.p(ix), O.p(d), C.byref(e))
    assert rc == 0, e.msg
    return ip, ix, d


def oracle_array_from_triplets(rows, cols, data, shape, sorted_):
    nnz = len(data)
    ip = np.empty(shape[0] + 1, dtype=np.uint64)
    ix = np.empty(nnz, dtype=np.uint64)
    d = np.empty(nnz, dtype=data.dtype)
    s, e = C.c_int(), O.Err()
    rc = O.lib().or_csr_array_from_triplets_f64(O.p(rows), O.p(cols), O.p(data), nnz, shape[0], shape[1],
                                                1 if sorted_ else 0, O.p(ip), O.p(ix), O.p(d), C.byref(s),
                                                C.byref(e))
    assert rc == 0, e.msg
    return ip, ix, d, bool(s.value)


def oracle_transpose(ip, ix, d, shape):
    tp = np.empty(shape[1] + 1, dtype=np.uint64)
    ti = np.empty(len(d), dtype=np.uint64)
    td = np.empty(len(d), dtype=d.dtype)
    f = O.lib().or_csr_transpose_f64 if d.dtype == np.float64 else O.lib().or_csr_transpose_f32
    f(O.p(ip), O.p(ix), O.p(d), shape[0], shape[1], O.p(tp), O.p(ti), O.p(td))
    return tp, ti, td


def random_triplets(rng, nrows, ncols, nnz, dup_frac=0.2, dtype=np.float64):
    rows = rng.integers(0, nrows, nnz).astype(np.uint64)
    cols = rng.integers(0, ncols, nnz).astype(np.uint64)
    ndup = int(nnz * dup_frac)
    if ndup:
        src = rng.integers(0, nnz, ndup)
        dst = rng.integers(0, nnz, ndup)
        rows[dst] = rows[src]
        cols[dst] = cols[src]
    data = rng.standard_normal(nnz).astype(dtype)
    return rows, cols, data


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape,nnz", [((1, 1), 1), ((7, 5), 40), ((300, 200), 5000), ((20000, 30000), 400000)])
def test_csr_matrix_new_bit_exact(S, ctx, dtype, shape, nnz):
    rng = np.random.default_rng(nnz)
    rows, cols, data = random_triplets(rng, *shape, nnz, dtype=dtype)
    a = S.csr_matrix(ctx, data, rows, cols, shape, dtype=dtype)
    ip, ix, d = a.to_arrays()
    rip, rix, rd = oracle_matrix_new(rows, cols, data, shape)
    assert np.array_equal(ip, rip) and np.array_equal(ix, rix)
    assert np.array_equal(d.view(np.uint8), rd.view(np.uint8))


def test_long_rows_and_sorted_flag(S, ctx):
    # rows longer than the in-shared-memory sort (2048) take the merge path
    rng = np.random.default_rng(5)
    nnz = 30000
    rows = np.concatenate([np.zeros(9000), rng.integers(0, 50, nnz - 9000)]).astype(np.uint64)
    cols = rng.integers(0, 4000, nnz).astype(np.uint64)
    data = rng.standard_normal(nnz)
    a = S.csr_matrix(ctx, data, rows, cols, (50, 4000))
    ip, ix, d = a.to_arrays()
    rip, rix, rd = oracle_matrix_new(rows, cols, data, (50, 4000))
    assert np.array_equal(ip, rip) and np.array_equal(ix, rix) and np.array_equal(d, rd)
    # CsrArray::from_triplets with sorted=true keeps the input order
    b = S.csr_array_from_triplets(ctx, rows, cols, data, (50, 4000), sorted=True)
    ip, ix, d = b.to_arrays()
    rip, rix, rd, rs = oracle_array_from_triplets(rows, cols, data, (50, 4000), True)
    assert np.array_equal(ip, rip) and np.array_equal(ix, rix) and np.array_equal(d, rd)
    assert b.has_sorted_indices == rs


@pytest.mark.parametrize("shape,nnz", [((5, 9), 30), ((3000, 2000), 60000)])
def test_transpose_bit_exact(S, ctx, shape, nnz):
    rng = np.random.default_rng(11)
    rows, cols, data = random_triplets(rng, *shape, nnz)
    a = S.csr_matrix(ctx, data, rows, cols, shape)
    ip, ix, d = a.to_arrays()
    t = a.transpose()
    tp, ti, td = t.to_arrays()
    rp, ri, rd = oracle_transpose(ip, ix, d, shape)
    assert t.shape == (shape[1], shape[0])
    assert np.array_equal(tp, rp) and np.array_equal(ti, ri) and np.array_equal(td, rd)
    # CsrArray::transpose goes through from_triplets(sorted=false): same arrays
    rip, rix, rd2, _ = oracle_array_from_triplets(ix.astype(np.uint64), np.repeat(np.arange(shape[0]), np.diff(ip.astype(np.int64))).astype(np.uint64), d, (shape[1], shape[0]), False)
    assert np.array_equal(rip, tp) and np.array_equal(rix, ti) and np.array_equal(rd2, td)


@pytest.mark.parametrize("kind,dims,dtype", [
    ("poisson2d", (256, 256, 1), np.float64),
    ("laplace3d", (32, 32, 32), np.float64),
    ("laplace3d", (32, 32, 32), np.float32),
    ("varcoef3d", (24, 20, 16), np.float64),
    ("aniso_q1", (64, 48, 1), np.float64),
    ("powerlaw", (20000, 1, 1), np.float64),
    ("powerlaw", (20000, 1, 1), np.float32),
])
def test_spmv_bit_exact(S, ctx, kind, dims, dtype):
    p0 = 1.5 if kind == "varcoef3d" else (100.0 if kind == "aniso_q1" else 0.0)
    p1 = 0.7 if kind == "aniso_q1" else 0.0
    if kind == "powerlaw":
        p0, p1 = 16.0, 4096.0
    ip, ix, v = S.generate(kind, *dims, seed=3, param0=p0, param1=p1)
    n = len(ip) - 1
    vals = v.astype(dtype)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    x = S.rhs_normal(9, n).astype(dtype)
    y = a.matvec(x)
    yr = O.spmv_i32(ip, ix, vals, x)
    assert np.array_equal(y.view(np.uint8), yr.view(np.uint8))


def _system(S, kind, dims, seed=1, p0=0.0, p1=0.0):
    ip, ix, v = S.generate(kind, *dims, seed=seed, param0=p0, param1=p1)
    n = len(ip) - 1
    return ip, ix, v, n, S.rhs_normal(seed + 100, n)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_cg_jacobi_matches_oracle(S, ctx, dtype):
    ip, ix, v, n, b = _system(S, "poisson2d", (64, 64, 1))
    vals = v.astype(dtype)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    m = S.jacobi(ctx, a)
    rtol = 1e-10 if dtype == np.float64 else 1e-5
    r = S.cg(a, b, max_iter=5000, rtol=rtol, atol=0.0, preconditioner=m)
    oa = O.op_csr_i32(ip, ix, v, (n, n), f64=dtype == np.float64)
    ro = O.cg(oa, b, max_iter=5000, rtol=rtol, atol=0.0, preconditioner=O.op_jacobi(oa))
    assert r.converged and ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= max(2, ro["iterations"] // 100)
    err = np.linalg.norm(r.x.astype(np.float64) - ro["x"]) / np.linalg.norm(ro["x"])
    assert err < (1e-8 if dtype == np.float64 else 1e-4)


def test_cg_unpreconditioned_and_x0(S, ctx):
    ip, ix, v, n, b = _system(S, "varcoef3d", (12, 10, 8), p0=1.0)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    x0 = np.linspace(-1, 1, n)
    r = S.cg(a, b, max_iter=3000, rtol=1e-10, atol=0.0, x0=x0)
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    ro = O.cg(oa, b, max_iter=3000, rtol=1e-10, atol=0.0, x0=x0)
    assert r.converged and abs(r.iterations - ro["iterations"]) <= 3
    assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-8


def test_cg_max_iter_path(S, ctx):
    ip, ix, v, n, b = _system(S, "poisson2d", (40, 40, 1))
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.cg(a, b, max_iter=7, rtol=1e-14, atol=0.0)
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    ro = O.cg(oa, b, max_iter=7, rtol=1e-14, atol=0.0)
    assert not r.converged and r.iterations == 7 == ro["iterations"]
    assert r.message == ro["message"] == "Maximum iterations reached"
    assert np.allclose(r.x, ro["x"], rtol=1e-12, atol=1e-12)
    assert np.isclose(r.residual_norm, ro["residual_norm"], rtol=1e-10)


@pytest.mark.parametrize("prec", ["none", "left", "right", "both"])
def test_bicgstab_matches_oracle(S, ctx, prec):
    # non-symmetric, diagonally dominant: convection on a variable-coefficient stencil
    ip, ix, v, n, b = _system(S, "varcoef2d", (40, 30, 1), p0=0.5)
    v = v.copy()
    for r in range(n):
        for k in range(ip[r], ip[r + 1]):
            if ix[k] == r + 1:
                v[k] *= 1.3
            if ix[k] == r:
                v[k] *= 1.5
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    m = S.jacobi(ctx, a)
    om = O.op_jacobi(oa)
    left = m if prec in ("left", "both") else None
    right = m if prec in ("right", "both") else None
    r = S.bicgstab(a, b, max_iter=2000, rtol=1e-8, atol=0.0, left_preconditioner=left,
                   right_preconditioner=right)
    ro = O.bicgstab(oa, b, max_iter=2000, rtol=1e-8, atol=0.0,
                    left=om if left else None, right=om if right else None)
    # with both, the reference's x = M2 x inside every iteration (iterative.rs:583-585)
    # derails the solve into a breakdown; the device must report the same
    assert r.converged == ro["converged"] and r.message == ro["message"]
    assert abs(r.iterations - ro["iterations"]) <= 2
    if ro["converged"]:
        assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-6


@pytest.mark.parametrize("restart,prec", [(30, False), (10, True), (500, False)])
def test_gmres_matches_oracle(S, ctx, restart, prec):
    ip, ix, v, n, b = _system(S, "varcoef2d", (24, 20, 1), p0=0.5)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    m = S.jacobi(ctx, a) if prec else None
    r = S.gmres(a, b, max_iter=3000, restart=restart, rtol=1e-10, atol=0.0, preconditioner=m)
    ro = O.gmres(oa, b, max_iter=3000, restart=restart, rtol=1e-10, atol=0.0,
                 preconditioner=O.op_jacobi(oa) if prec else None)
    assert r.converged and ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= max(3, ro["iterations"] // 20)
    assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-8


def test_mixed_precision_refinement(S, ctx):
    ip, ix, v, n, b = _system(S, "varcoef3d", (24, 24, 24), p0=1.5)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.cg_mixed(a, b, tol=1e-10, inner_rtol=1e-4, mode="restart")
    assert r.converged and r.rel_residual <= 1e-10
    res = O.true_rel_residual(ip, ix, v, b, r.x)
    assert res <= 1.5e-10
    ro = O.cg_mixed_ir(ip, ix, v, b, tol=1e-10, inner_rtol=1e-4)
    assert ro["converged"]
    # both solve to 1e-10: the solutions agree to ~cond * 1e-10
    assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-7
    assert abs(S.true_rel_residual(a, b, r.x) - res) <= 1e-3 * res


@pytest.mark.parametrize("kind,dims,p0,p1,tol", [
    ("varcoef3d", (24, 24, 24), 1.5, 0.0, 1e-10),
    ("aniso_q1", (96, 80, 1), 500.0, 0.6, 1e-8),
    ("laplace3d", (40, 40, 40), 0.0, 0.0, 1e-10),
])
def test_mixed_precision_residual_replacement(S, ctx, kind, dims, p0, p1, tol):
    ip, ix, v, n, b = _system(S, kind, dims, p0=p0, p1=p1)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.cg_mixed(a, b, tol=tol, mode="replace")
    assert r.converged and r.rel_residual <= tol
    res = O.true_rel_residual(ip, ix, v, b, r.x)
    assert res <= 1.5 * tol
    ro = O.cg_mixed_replace(ip, ix, v, b, tol=tol)
    assert ro["converged"]
    # the same algorithm: FP32 rounding of the reductions differs, the
    # iteration counts stay close
    assert abs(r.inner_iterations - ro["inner"]) <= 0.15 * ro["inner"] + 5, (r.inner_iterations, ro["inner"])
    # fewer FP32 iterations than restarted refinement
    rr = S.cg_mixed(a, b, tol=tol, inner_rtol=1e-4, mode="restart")
    assert r.inner_iterations <= rr.inner_iterations
    assert np.linalg.norm(r.x - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-5


def test_host_operator_and_rmatvec(S, ctx):
    ip, ix, v, n, b = _system(S, "poisson2d", (10, 10, 1))
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    dense = np.zeros((n, n))
    for r in range(n):
        dense[r, ix[ip[r]:ip[r + 1]]] = v[ip[r]:ip[r + 1]]
    h = S.host_operator(ctx, n, lambda x: dense @ x)
    r = S.cg(h, b, max_iter=500, rtol=1e-10, atol=0.0)
    r2 = S.cg(a, b, max_iter=500, rtol=1e-10, atol=0.0)
    assert r.converged and np.allclose(r.x, r2.x, rtol=1e-8, atol=1e-10)
    x = np.arange(n, dtype=np.float64)
    assert np.allclose(a.rmatvec(x), dense.T @ x)


def test_preconditioners_rebuilt_from_one_matrix(S, ctx):
    # a fresh Jacobi / IC(0) operator per solve over one matrix: each solve
    # captures its own graph and gets the same answer
    ip, ix, v, n, b = _system(S, "poisson2d", (60, 50, 1))
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    out = []
    for _ in range(3):
        m = S.jacobi(ctx, a)
        r = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=m)
        m.close()
        out.append((r.iterations, r.x.copy()))
    for it, x in out[1:]:
        assert it == out[0][0] and np.array_equal(x, out[0][1])
    # a bigger system in between grows the reduction area; the same pair
    # (a, m) solves before and after it
    m = S.jacobi(ctx, a)
    r = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=m)
    assert r.iterations == out[0][0]
    ip2, ix2, v2, n2, b2 = _system(S, "laplace3d", (300, 250, 200))
    a2 = S.csr_from_arrays(ctx, ip2, ix2, v2, (n2, n2))
    m2 = S.jacobi(ctx, a2)
    S.cg(a2, b2, max_iter=3, rtol=1e-10, atol=0.0, preconditioner=m2)
    m2.close()
    a2.close()
    r = S.cg(a, b, max_iter=2000, rtol=1e-10, atol=0.0, preconditioner=m)
    assert r.iterations == out[0][0] and np.array_equal(r.x, out[0][1])
    m.close()
    a.close()


def _ctx_env(S, env):
    import os
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


@pytest.mark.parametrize("kind,dims,p0,p1", [
    ("aniso_q1", (128, 96, 1), 300.0, 0.6),
    ("laplace3d", (40, 36, 32), 0.0, 0.0),
])
@pytest.mark.parametrize("short", ["0", "2"])
def test_fused_replacement_loop_matches_plain_kernels(S, kind, dims, p0, p1, short):
    # the fused FP32 iteration (q = A z + beta q, x/r updates in the SpMV
    # epilogues) against the plain CG kernels: same algorithm, FP32 rounding
    # apart; both reach the FP64 target
    ip, ix, v, n, b = _system(S, kind, dims, p0=p0, p1=p1)
    res = {}
    for mode in ("1", "0"):
        c = _ctx_env(S, {"SX_MX_FUSED": mode, "SX_SHORT": short})
        a = S.csr_from_arrays(c, ip, ix, v, (n, n))
        r = S.cg_mixed(a, b, tol=1e-9)
        assert r.converged and O.true_rel_residual(ip, ix, v, b, r.x) <= 1.5e-9
        res[mode] = r.inner_iterations
        a.close()
        c.close()
    assert abs(res["1"] - res["0"]) <= 0.1 * res["0"] + 3, res


@pytest.mark.parametrize("short", ["0", "2"])
def test_fused_replacement_loop_with_factored_preconditioner(S, short):
    # M = G G^T (FSAI operator): the fused G^T / G steps against the plain ones
    ip, ix, v, n, b = _system(S, "aniso_q1", (100, 90, 1), p0=50.0, p1=1.2)
    # G = D^-1/2 on the lower pattern (a Jacobi-like factor with the full pattern)
    lens, cols, vals = [], [], []
    for i in range(n):
        row = ix[ip[i]:ip[i + 1]]
        low = row[row < i]
        d = v[ip[i]:ip[i + 1]][row == i][0]
        cols.append(np.concatenate([low, [i]]))
        vals.append(np.concatenate([np.full(len(low), -0.05 / np.sqrt(d)), [1.0 / np.sqrt(d)]]))
        lens.append(len(low) + 1)
    gp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    gi = np.concatenate(cols).astype(np.int32)
    gv = np.concatenate(vals).astype(np.float32)
    res = {}
    for mode in ("1", "0"):
        c = _ctx_env(S, {"SX_MX_FUSED": mode, "SX_SHORT": short})
        a = S.csr_from_arrays(c, ip, ix, v, (n, n))
        a32 = a.astype(np.float32)
        G = S.csr_from_arrays(c, gp, gi, gv, (n, n))
        m = S.fsai(c, G)
        r = S.cg_mixed(a, b, tol=1e-9, preconditioner=m, a32=a32)
        assert r.converged and O.true_rel_residual(ip, ix, v, b, r.x) <= 1.5e-9
        res[mode] = r.inner_iterations
        for op in (m, G, a32, a):
            op.close()
        c.close()
    assert abs(res["1"] - res["0"]) <= 0.1 * res["0"] + 3, res
