"""save_npz / load_npz through the device library (io.rs:49-269).

The reference's io tests (identity and random round trips, io.rs:350-436),
byte equality of saved files with the restated record layout, loading of
records written by the restatement (including FP32 widths and the CsrArray
validation), and the reference's error texts for missing, short, mislabelled
and non-UTF-8 files.
"""
import errno
import os

import numpy as np
import pytest

from oracle import npz_format as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def test_identity_round_trip(S, ctx, tmp_path):
    # io.rs:350-374
    eye = S.csr_array_from_triplets(ctx, list(range(5)), list(range(5)), [1.0] * 5, (5, 5))
    p = tmp_path / "test_csr.npz"
    S.save_npz(eye, p)
    loaded = S.load_npz(ctx, p)
    assert loaded.shape == (5, 5) and loaded.nnz == 5
    for i in range(5):
        assert loaded.get(i, i) == 1.0
    assert loaded.get(0, 1) == 0.0
    assert p.read_bytes() == N.record("csr_array", (5, 5), np.ones(5), np.arange(5), np.arange(6))


def test_random_round_trip_and_bytes(S, ctx, tmp_path):
    # io.rs:402-436 (nnz and sum survive), plus bit-identical arrays
    rng = np.random.default_rng(42)
    for dt in (np.float64, np.float32):
        ip, ix, v = S.generate("powerlaw", 5000, seed=3, param0=6.0, param1=200.0)
        n = len(ip) - 1
        a = S.csr_from_arrays(ctx, ip, ix, v.astype(dt), (n, n + 7))
        p = tmp_path / f"rand_{np.dtype(dt).name}.npz"
        S.save_npz(a, p)
        assert p.read_bytes() == N.record("csr_array", (n, n + 7), v.astype(dt), ix, ip, dtype=dt)
        b = S.load_npz(ctx, p, dtype=dt)
        assert b.shape == (n, n + 7) and b.nnz == len(v)
        ip2, ix2, v2 = b.to_arrays()
        assert np.array_equal(ip2, ip) and np.array_equal(ix2, ix) and np.array_equal(v2, v.astype(dt))
        x = rng.standard_normal(n + 7).astype(dt)
        assert np.array_equal(a.matvec(x), b.matvec(x))


def test_load_restated_records(S, ctx, tmp_path):
    p = tmp_path / "r.npz"
    # unsorted columns are kept as stored (CsrArray::new)
    p.write_bytes(N.record("csr_array", (2, 3), [1.0, 2.0, 3.0], [2, 0, 1], [0, 2, 3]))
    a = S.load_npz(ctx, p)
    assert a.shape == (2, 3) and a.nnz == 3 and not a.has_sorted_indices
    assert a.get(0, 2) == 1.0 and a.get(0, 0) == 2.0 and a.get(1, 1) == 3.0
    # a record loaded at the other width reads the value bytes as that type
    p.write_bytes(N.record("csr_array", (1, 2), [1.0, 2.0], [0, 1], [0, 2], dtype=np.float32))
    a = S.load_npz(ctx, p, dtype=np.float32)
    assert a.get(0, 1) == np.float32(2.0)
    # CsrArray::new's checks
    p.write_bytes(N.record("csr_array", (2, 2), [1.0, 2.0], [0], [0, 1, 1]))
    with pytest.raises(S.SparseError, match="Inconsistent data: data and indices must have the same length"):
        S.load_npz(ctx, p)
    p.write_bytes(N.record("csr_array", (2, 2), [1.0], [0], [0, 1]))
    with pytest.raises(S.SparseError, match=r"Inconsistent data: indptr length \(2\) must be one more than the number of rows \(2\)"):
        S.load_npz(ctx, p)
    p.write_bytes(N.record("csr_array", (2, 2), [1.0], [5], [0, 1, 1]))
    with pytest.raises(S.SparseError, match=r"Index \(0, 5\) out of bounds for array with shape \(2, 2\)"):
        S.load_npz(ctx, p)


def test_error_texts(S, ctx, tmp_path):
    missing = tmp_path / "none.npz"
    with pytest.raises(S.SparseError) as e:
        S.load_npz(ctx, missing)
    assert str(e.value) == f"Computation error: IO error: {os.strerror(errno.ENOENT)} (os error {errno.ENOENT})"
    p = tmp_path / "short.npz"
    full = N.record("csr_array", (5, 5), np.ones(5), np.arange(5), np.arange(6))
    for cut in (3, 20, len(full) - 1):
        p.write_bytes(full[:cut])
        with pytest.raises(S.SparseError, match="Computation error: IO error: failed to fill whole buffer"):
            S.load_npz(ctx, p)
    p.write_bytes(N.record("bsr_array", (1, 1), [1.0], [0], [0, 1]))
    with pytest.raises(S.SparseError, match="Conversion error: Unknown format: bsr_array"):
        S.load_npz(ctx, p)
    p.write_bytes(N.record("coo_array", (1, 1), [1.0], [0], [0]))
    with pytest.raises(S.SparseError, match="Feature not implemented"):
        S.load_npz(ctx, p)
    p.write_bytes(N.record(b"csr\xffarray", (1, 1), [1.0], [0], [0, 1]))
    with pytest.raises(S.SparseError, match="Computation error: IO error: invalid utf-8 sequence of 1 bytes from index 3"):
        S.load_npz(ctx, p)
    p.write_bytes(N.record(b"csr\xe2\x82", (1, 1), [1.0], [0], [0, 1]))
    with pytest.raises(S.SparseError, match="Computation error: IO error: incomplete utf-8 byte sequence from index 3"):
        S.load_npz(ctx, p)
    # a length field far beyond the file reads as an early end of file
    p.write_bytes(N.record("csr_array", (1, 1), [1.0], [0], [0, 1])[:33] + (2**62).to_bytes(8, "little"))
    with pytest.raises(S.SparseError, match="failed to fill whole buffer"):
        S.load_npz(ctx, p)
    with pytest.raises(S.SparseError, match="IO error"):
        S.save_npz(S.csr_array_from_triplets(ctx, [0], [0], [1.0], (1, 1)), tmp_path / "no_such_dir" / "x.npz")
