"""Parity on the benchmark's own configurations, against the oracle (GPU).

Each test runs one benchmark configuration at its full size through the C
ABI and checks the device's answer with the oracle's restatement of the
reference (iterative.rs:40-162, csr.rs:479-497, csr_array.rs:569-593,
index_dtype.rs:109-170):

- 2D 5-point Poisson 256^2, FP64 Jacobi-PCG, rtol 1e-8, maxiter 5000: the
  same exit and message, iterations within 2, solutions within 1e-8 relative
  at the solver's rtol of 1e-10;
- the headline 1024^2 anisotropic Q1 problem: the learned mixed-precision
  solve reaches the oracle's FP64 true residual of 1e-8; FP64 Jacobi-PCG
  takes the oracle's iteration count (within 2) and its iterate after 300
  steps matches the oracle's;
- the 4M-row power-law SpMV in FP64 and FP32: bit-exact, and the FP64
  fused-multiply-add mode within (len + 1) eps sum|a x| per row;
- 3D variable-coefficient diffusion 160^3, mixed precision to 1e-10: the
  oracle's FP64 true residual <= 1.5e-10;
- batched PCG on systems with sides drawn from [32, 256]: every system's
  oracle residual <= 1e-8;
- indices beyond i32::MAX: IndexCastOverflow with the first offending value.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADLINE_SEED = 1000001


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


@pytest.fixture(scope="module", autouse=True)
def oracle_threads():
    # row-parallel oracle loops (bit-identical to one thread) keep the
    # full-size oracle solves to seconds
    old = O.get_threads()
    O.set_threads(len(os.sched_getaffinity(0)))
    yield
    O.set_threads(old)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("rtol", [1e-8, 1e-10])
def test_poisson256_jacobi_pcg_fp64(S, ctx, rtol):
    ip, ix, v = S.generate("poisson2d", 256, 256)
    n = len(ip) - 1
    assert n == 65536 and len(v) == 326656
    b = S.rhs_normal(0, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    m = S.jacobi(ctx, a)
    r = S.cg(a, b, max_iter=5000, rtol=rtol, atol=0.0, preconditioner=m)
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    ro = O.cg(oa, b, max_iter=5000, rtol=rtol, atol=0.0, preconditioner=O.op_jacobi(oa))
    assert r.converged and ro["converged"]
    assert r.message == ro["message"]
    assert abs(r.iterations - ro["iterations"]) <= 2
    if rtol == 1e-10:
        assert _rel(r.x, ro["x"]) <= 1e-8
    assert O.true_rel_residual(ip, ix, v, b, r.x) <= rtol * 1.01
    m.close()
    a.close()


@pytest.fixture(scope="module")
def headline(S, ctx):
    from scirs_gb300 import learned as LR

    p = LR.sample_problem(HEADLINE_SEED)
    ip, ix, v = S.generate("aniso_q1", 1024, 1024, param0=p.eps, param1=p.theta)
    n = len(ip) - 1
    b = S.rhs_normal(HEADLINE_SEED, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    yield ip, ix, v, n, b, a
    a.close()


def test_headline_learned_solve_oracle_residual(S, ctx, headline):
    from scirs_gb300 import learned as LR

    ip, ix, v, n, b, a = headline
    assert n == 1048576 and len(v) == 9424900
    net = LR.load_weights(ctx, os.path.join(REPO, "scirs_gb300", "weights", "aniso_q1.npz"))
    try:
        r = LR.solve(net, a, b, tol=1e-8)
    finally:
        net.close()
    assert r.converged and r.method == "learned-mixed"
    res = O.true_rel_residual(ip, ix, v, b, r.x)
    assert res <= 1e-8 * (1 + 1e-6), res
    assert abs(res - r.rel_residual) <= 1e-6 * res


def test_headline_jacobi_pcg_fp64_matches_oracle(S, ctx, headline):
    ip, ix, v, n, b, a = headline
    m = S.jacobi(ctx, a)
    oa = O.op_csr_i32(ip, ix, v, (n, n))
    om = O.op_jacobi(oa)
    # the iterate after a fixed number of steps
    r300 = S.cg(a, b, max_iter=300, rtol=1e-8, atol=0.0, preconditioner=m)
    o300 = O.cg(oa, b, max_iter=300, rtol=1e-8, atol=0.0, preconditioner=om)
    assert r300.iterations == o300["iterations"] == 300 and not r300.converged
    # the device's solver-internal SpMV fuses multiply-adds: rounding, not
    # the method, separates the two iterates
    assert _rel(r300.x, o300["x"]) <= 1e-8
    assert abs(r300.residual_norm - o300["residual_norm"]) <= 1e-6 * o300["residual_norm"]
    # the complete solve
    r = S.cg(a, b, max_iter=200000, rtol=1e-8, atol=0.0, preconditioner=m)
    ro = O.cg(oa, b, max_iter=200000, rtol=1e-8, atol=0.0, preconditioner=om)
    assert r.converged and ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= 2, (r.iterations, ro["iterations"])
    assert O.true_rel_residual(ip, ix, v, b, r.x) <= 1e-8 * 1.01
    m.close()


@pytest.fixture(scope="module")
def powerlaw(S):
    ip, ix, v = S.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0)
    return ip, ix, v


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_powerlaw_4m_spmv_bit_exact(S, ctx, powerlaw, dtype):
    ip, ix, v = powerlaw
    n = len(ip) - 1
    assert n == 4194304 and np.diff(ip).max() <= 4096
    vals = v.astype(dtype)
    a = S.csr_from_arrays(ctx, ip, ix, vals, (n, n))
    x = S.rhs_normal(9, n).astype(dtype)
    y = a.matvec(x)
    yr = O.spmv_i32(ip, ix, vals, x)
    assert np.array_equal(y.view(np.uint8), yr.view(np.uint8))
    a.close()


def test_powerlaw_4m_spmv_fp64_fma_within_bound(S, ctx, powerlaw):
    import torch

    from scirs_gb300 import _lib as L

    ip, ix, v = powerlaw
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    x = S.rhs_normal(10, n)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, a.handle, C.c_void_p(xd.data_ptr()),
                                     C.c_void_p(yd.data_ptr()), 0))
    ctx.synchronize()
    y = yd.cpu().numpy()
    yr = O.spmv_i32(ip, ix, v, x)
    lens = np.diff(ip)
    mag = np.add.reduceat(np.abs(v * x[ix]), ip[:-1]) if len(v) else np.zeros(n)
    mag[lens == 0] = 0.0
    bound = (lens + 1.0) * np.finfo(np.float64).eps * mag
    assert np.all(np.abs(y - yr) <= bound + 1e-300)
    a.close()


def test_varcoef160_mixed_oracle_residual(S, ctx):
    ip, ix, v = S.generate("varcoef3d", 160, 160, 160, seed=0, param0=1.5)
    n = len(ip) - 1
    assert n == 4096000 and len(v) == 28518400
    b = S.rhs_normal(0, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    a32 = a.astype(np.float32)
    m32 = S.jacobi(ctx, a32)
    r = S.cg_mixed(a, b, tol=1e-10, max_inner=100000, preconditioner=m32, a32=a32)
    assert r.converged
    res = O.true_rel_residual(ip, ix, v, b, r.x)
    assert res <= 1.5e-10, res
    assert abs(res - r.rel_residual) <= 1e-4 * res
    for op in (m32, a32, a):
        op.close()


def test_batched_sides_32_to_256(S, ctx):
    sp, ip, ix, v = S.generate_batch(64, 32, 256, seed=3, sigma=1.0)
    sides = np.sqrt(np.diff(sp)).astype(np.int64)
    assert sides.min() >= 32 and sides.max() <= 256 and sides.max() - sides.min() > 150
    n = len(ip) - 1
    b = S.rhs_normal(5, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.batched_pcg(a, sp, b, rtol=1e-8)
    assert r.converged.all()
    for s in range(len(sp) - 1):
        r0, r1 = sp[s], sp[s + 1]
        k0, k1 = ip[r0], ip[r1]
        res = O.true_rel_residual(ip[r0:r1 + 1] - k0, ix[k0:k1] - r0, v[k0:k1], b[r0:r1], r.x[r0:r1])
        assert res <= 1e-8 * 1.0001, (s, sides[s], res)
        assert abs(res - r.rel_residual[s]) <= 1e-3 * res + 1e-16
    a.close()


def test_index_cast_overflow(S, ctx):
    big = 3_000_000_000  # > i32::MAX
    # a triplet whose row index does not fit: IndexCastOverflow with that value
    # (CsrMatrix::new takes data, rows, cols; CsrArray::from_triplets rows, cols, data)
    calls = (lambda: S.csr_matrix(ctx, [1.0, 2.0], [0, big], [0, 1], (4_000_000_000, 4)),
             lambda: S.csr_array_from_triplets(ctx, [0, big], [0, 1], [1.0, 2.0], (4_000_000_000, 4)))
    for call in calls:
        with pytest.raises(S.SparseError) as e:
            call()
        assert e.value.variant == "IndexCastOverflow" and e.value.payload[0] == big
        assert f"Index value {big} cannot be represented" in e.value.message
    # a column index that does not fit, through the raw constructors
    with pytest.raises(S.SparseError) as e:
        S.csr_matrix_from_raw(ctx, [1.0, 2.0], [0, 1, 2], [5, big], (2, 4_000_000_000))
    assert e.value.variant == "IndexCastOverflow" and e.value.payload[0] == big
    with pytest.raises(S.SparseError) as e:
        S.csr_array(ctx, [1.0, 2.0], [5, big], [0, 1, 2], (2, 4_000_000_000))
    assert e.value.variant == "IndexCastOverflow" and e.value.payload[0] == big
    # small indices but a row count beyond i32: the dimension is the value
    with pytest.raises(S.SparseError) as e:
        S.csr_matrix(ctx, [1.0], [0], [0], (3_000_000_000, 3))
    assert e.value.variant == "IndexCastOverflow" and e.value.payload[0] == 3_000_000_000
    # the largest values that fit are accepted
    a = S.csr_array_from_triplets(ctx, [2], [2**31 - 2], [1.0], (3, 2**31 - 1))
    assert a.nnz == 1
    a.close()
