"""Oracle restatement of SymCsrMatrix / sym_ops pinned on the reference's tests.

Known answers come from scirs2-sparse/src/sym_csr.rs:498-593 (creation,
from_csr, to_csr), src/sym_ops.rs:348-459 (matvec, rank-1 update, quadratic
form, trace) and src/test_dimension_mismatch.rs:5-33 (from_csr of a
non-symmetric matrix).  Property checks compare the restated loops with
dense numpy arithmetic at tolerance.
"""
import numpy as np
import pytest

from oracle import oracle_ffi as O

# sym_csr.rs:510-512 / sym_ops.rs:357-359: lower part of [[2,1,0],[1,2,3],[0,3,1]]
DATA = np.array([2.0, 1.0, 2.0, 3.0, 1.0])
INDICES = np.array([0, 0, 1, 1, 2])
INDPTR = np.array([0, 1, 3, 5])


def test_creation_known_answers():
    assert O.sym_check(5, INDPTR, INDICES, (3, 3)) == (0, "")
    assert O.sym_nnz(INDPTR, INDICES) == 7  # sym_csr.rs:520
    expect = {(0, 0): 2.0, (0, 1): 1.0, (1, 0): 1.0, (1, 1): 2.0, (1, 2): 3.0, (2, 1): 3.0}
    for (i, j), v in expect.items():  # sym_csr.rs:523-528
        assert O.sym_get(INDPTR, INDICES, DATA, i, j) == v
    assert O.sym_get(INDPTR, INDICES, DATA, 0, 2) == 0.0
    assert O.sym_get(INDPTR, INDICES, DATA, 5, 0) == 0.0


def test_matvec_quadratic_trace_known_answers():
    x = np.array([1.0, 2.0, 3.0])
    assert list(O.sym_matvec(INDPTR, INDICES, DATA, x)) == [4.0, 14.0, 9.0]  # sym_ops.rs:395-398
    assert O.sym_quadratic_form(INDPTR, INDICES, DATA, x) == 59.0  # sym_ops.rs:433
    assert O.sym_trace(INDPTR, INDICES, DATA) == 5.0  # sym_ops.rs:443
    y32 = O.sym_matvec(INDPTR, INDICES, DATA.astype(np.float32), x.astype(np.float32))
    assert y32.dtype == np.float32 and list(y32) == [4.0, 14.0, 9.0]


def test_rank1_update_known_answer():
    ip, ix, dv = O.sym_rank1_update(INDPTR, INDICES, DATA, np.array([1.0, 0.0, 0.0]), 3.0)
    get = lambda i, j: O.sym_get(ip, ix, dv, i, j)  # noqa: E731
    assert get(0, 0) == 5.0  # sym_ops.rs:412
    assert (get(0, 1), get(1, 1), get(1, 2), get(2, 2)) == (1.0, 2.0, 3.0, 1.0)  # :415-418


def test_from_csr_known_answers():
    # sym_csr.rs:542-546: CsrMatrix::new of the full symmetric matrix
    ip = np.array([0, 2, 5, 7])
    ix = np.array([0, 1, 0, 1, 2, 1, 2])
    dv = np.array([2.0, 1.0, 1.0, 2.0, 3.0, 3.0, 1.0])
    (lp, li, lv), err = O.sym_from_csr(ip, ix, dv, (3, 3))
    assert err is None
    assert list(lp) == [0, 1, 3, 5] and list(li) == [0, 0, 1, 1, 2] and list(lv) == list(DATA)
    # test_dimension_mismatch.rs:7-9: (2, 0) = 3 has no (0, 2) partner
    ip2 = np.array([0, 2, 4, 7])
    ix2 = np.array([0, 1, 0, 1, 0, 1, 2])
    res, err = O.sym_from_csr(ip2, ix2, dv, (3, 3))
    assert res is None and err == "Value error: Matrix must be symmetric to convert to SymCSR format"
    _, err = O.sym_from_csr(ip, ix, dv, (3, 4))
    assert err == "Value error: Symmetric matrix must be square"


VALIDATION_CASES = [
        ((5, INDPTR, INDICES, (3, 4)), "Value error: Symmetric matrix must be square"),
        ((5, [0, 1, 3], INDICES, (3, 3)), "Value error: indptr length (3) must be equal to rows + 1 (4)"),
        ((4, INDPTR, INDICES, (3, 3)), "Value error: data length (4) must match indices length (5)"),
        ((5, [0, 1, 3, 4], INDICES, (3, 3)), "Value error: Last indptr value (4) must equal nnz (5)"),
        ((5, INDPTR, [0, 0, 1, 1, 3], (3, 3)), "Index (2, 3) out of bounds for array with shape (3, 3)"),
        ((5, INDPTR, [0, 0, 2, 1, 1], (3, 3)),
         "Value error: Symmetric CSR should only store the lower triangular part"),
        ((5, INDPTR, [1, 0, 1, 1, 2], (3, 3)),
         "Value error: Symmetric CSR should only store the lower triangular part"),
    ]


@pytest.mark.parametrize("args,msg", VALIDATION_CASES)
def test_validation_messages(args, msg):
    rc, m = O.sym_check(*args)
    assert rc != 0 and m == msg


def random_lower(rng, n, max_len=8, dup=True):
    """Lower-triangular CSR arrays with unsorted columns and duplicates."""
    lens = rng.integers(0, max_len + 1, n)
    if not dup:
        lens = np.minimum(lens, np.arange(1, n + 1))
    ip = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    ix = np.empty(int(ip[-1]), dtype=np.uint64)
    for i in range(n):
        s, e = int(ip[i]), int(ip[i + 1])
        cols = rng.integers(0, i + 1, e - s)
        if not dup:
            cols = rng.permutation(np.arange(i + 1))[: e - s]
        ix[s:e] = cols
    dv = rng.uniform(-1.0, 1.0, int(ip[-1]))
    return ip, ix, dv


def dense_of(ip, ix, dv, n):
    d = np.zeros((n, n))
    for i in range(n):
        for k in range(int(ip[i]), int(ip[i + 1])):
            j = int(ix[k])
            d[i, j] += dv[k]
            if i != j:
                d[j, i] += dv[k]
    return d


def test_matvec_matches_dense_sum():
    rng = np.random.default_rng(7)
    n = 200
    ip, ix, dv = random_lower(rng, n)
    x = rng.standard_normal(n)
    y = O.sym_matvec(ip, ix, dv, x)
    ref = dense_of(ip, ix, dv, n) @ x
    assert np.allclose(y, ref, rtol=1e-12, atol=1e-12)
    q = O.sym_quadratic_form(ip, ix, dv, x)
    assert abs(q - x @ ref) <= 1e-10 * (1 + abs(q))


def test_rank1_update_matches_dense():
    rng = np.random.default_rng(8)
    n = 40
    ip, ix, dv = random_lower(rng, n, dup=False)
    x = rng.standard_normal(n)
    x[rng.integers(0, n, 10)] = 0.0
    nip, nix, ndv = O.sym_rank1_update(ip, ix, dv, x, 0.5)
    full = dense_of(ip, ix, dv, n) + 0.5 * np.outer(x, x)
    got = dense_of(nip, nix, ndv, n)
    assert np.allclose(got, full, rtol=1e-14, atol=1e-14)
    assert np.all(ndv != 0.0)
    for i in range(n):  # columns ascending within each row
        row = nix[int(nip[i]):int(nip[i + 1])]
        assert np.all(np.diff(row.astype(np.int64)) > 0)
