"""The library's host tridiagonal eigensolver (the scalar step of lanczos,
eigen.rs:512-952) against the oracle's restatement, on the CPU: values and
eigenvectors bit for bit (both are plain FP64 host code without contraction),
and the same errors."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_ffi as O


def _lib_tridiag(alpha, beta, num):
    from scirs_gb300 import _lib as L
    from scirs_gb300 import sparse as S

    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    m = len(alpha)
    cap = max(1, min(num, max(m, 1)), 3)
    vals = np.zeros(cap)
    vecs = np.zeros(cap * max(m, 1))
    cnt = C.c_uint64()
    S._check(L.lib.sx_tridiag_eig(S._ptr(alpha) if m else None, S._ptr(beta) if len(beta) else None, m, len(beta),
                                  num, S._ptr(vals), S._ptr(vecs), C.byref(cnt)))
    c = int(cnt.value)
    return vals[:c], [vecs[k * m:(k + 1) * m] for k in range(c)]


def _cases():
    rng = np.random.default_rng(21)
    yield [3.0], [], 1
    yield [2.0, 1.0], [1.0], 2
    yield [2.0, 1.0], [0.0], 1
    yield [1.0, 0.0], [0.0], 2
    yield [1.0, 1.0, 1.0], [1.0, 1.0], 3
    yield [2.0, 0.0, -72.0], [1.0, 1.0], 3
    yield [2.0, 1.0, 3.0, 4.0], [0.0, 0.0, 0.0], 4
    yield [2.0, 1.0, 3.0, 4.0, 5.0], [1e-13, 0.0, 0.0, 0.0], 2
    for m in (2, 3):
        for _ in range(20):
            a = rng.standard_normal(m) * 4.0
            b = rng.standard_normal(m - 1)
            yield a, b, int(rng.integers(1, m + 1))


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def test_matches_oracle_bit_for_bit():
    for alpha, beta, num in _cases():
        try:
            ov, ovec = O.tridiag_eig(alpha, beta, num)
        except O.OracleError as e:
            from scirs_gb300 import sparse as S

            with pytest.raises(S.SparseError) as d:
                _lib_tridiag(alpha, beta, num)
            assert str(d.value) == str(e), (alpha, beta)
            continue
        dv, dvec = _lib_tridiag(alpha, beta, num)
        assert np.array_equal(_bits(dv), _bits(ov)), (alpha, beta, num, dv, ov)
        assert len(dvec) == len(ovec)
        for x, y in zip(dvec, ovec):
            assert np.array_equal(_bits(x), _bits(y)), (alpha, beta, num)


def test_errors():
    from scirs_gb300 import sparse as S

    with pytest.raises(S.SparseError, match="QL algorithm did not converge") as e:
        _lib_tridiag([2.0, 1.0, 3.0, 4.0], [1.0, 1.0, 1.0], 2)
    assert e.value.code == 13
    with pytest.raises(S.SparseError, match="Empty tridiagonal matrix"):
        _lib_tridiag([], [], 1)
    with pytest.raises(S.SparseError, match="Dimension mismatch: expected 1, found 2"):
        _lib_tridiag([1.0, 2.0], [1.0, 2.0], 1)
