"""The oracle's restatement of the workload generators against the library's
own (CPU).  The benchmark's reference arm builds its inputs with the oracle
so that it never loads the device library; both must give the same arrays
bit for bit, and the oracle's threaded loops must give the same solve as one
thread."""
import numpy as np
import pytest

from oracle import oracle_ffi as O

S = pytest.importorskip("scirs_gb300")


CASES = [
    ("poisson2d", (37, 29), {}),
    ("laplace3d", (13, 11, 9), {}),
    ("varcoef3d", (17, 13, 11), dict(seed=3, param0=1.5)),
    ("varcoef2d", (40, 33), dict(seed=9, param0=1.0)),
    ("aniso_q1", (45, 39), dict(param0=845.08, param1=0.9632)),
    ("aniso_q1", (1, 7), dict(param0=3.0, param1=0.1)),
    ("powerlaw", (50000,), dict(seed=1, param0=16.0, param1=4096.0)),
    ("powerlaw", (300,), dict(seed=4, param0=5.0, param1=64.0)),
]


@pytest.mark.parametrize("kind,dims,kw", CASES)
def test_generators_bit_identical(kind, dims, kw):
    a = S.generate(kind, *dims, **kw)
    b = O.generate(kind, *dims, **kw)
    for x, y in zip(a, b):
        assert x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_large_varcoef_and_rhs_bit_identical():
    # more than one 4096-value stream block, and the thread split of the library
    a = S.generate("varcoef3d", 70, 70, 70, seed=3, param0=1.5)
    b = O.generate("varcoef3d", 70, 70, 70, seed=3, param0=1.5)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert np.array_equal(S.rhs_normal(5, 300001).view(np.uint8), O.rhs_normal(5, 300001).view(np.uint8))


def test_batch_systems_bit_identical():
    sp, ip, ix, v = S.generate_batch(6, 32, 256, seed=0, sigma=1.0)
    sides = O.batch_sides(6, 32, 256, 0)
    assert np.array_equal(np.diff(sp), sides ** 2)
    for s in range(6):
        i2, x2, v2 = O.batch_system(s, int(sides[s]), 0, 1.0)
        r0, r1 = sp[s], sp[s + 1]
        k0, k1 = ip[r0], ip[r1]
        assert np.array_equal(ip[r0:r1 + 1] - k0, i2)
        assert np.array_equal(ix[k0:k1] - r0, x2)
        assert np.array_equal(v[k0:k1], v2)


def test_headline_problem_parameters():
    from scirs_gb300 import learned as LR

    p = LR.sample_problem(1000001)
    assert O.sample_problem(1000001) == (p.side, p.eps, p.theta)


def test_threaded_oracle_cg_bit_identical():
    ip, ix, v = O.generate("varcoef2d", 90, 70, seed=2, param0=1.0)
    n = len(ip) - 1
    b = O.rhs_normal(4, n)
    a = O.op_csr_i32(ip, ix, v, (n, n))
    m = O.op_jacobi(a)
    old = O.get_threads()
    try:
        O.set_threads(1)
        r1 = O.cg(a, b, max_iter=3000, rtol=1e-10, atol=0.0, preconditioner=m)
        O.set_threads(4)
        r4 = O.cg(a, b, max_iter=3000, rtol=1e-10, atol=0.0, preconditioner=m)
        y4 = O.spmv_i32(ip, ix, v, b)
        O.set_threads(1)
        y1 = O.spmv_i32(ip, ix, v, b)
    finally:
        O.set_threads(old)
    assert r1["iterations"] == r4["iterations"] and r1["converged"]
    assert np.array_equal(r1["x"].view(np.uint8), r4["x"].view(np.uint8))
    assert np.array_equal(y1.view(np.uint8), y4.view(np.uint8))
