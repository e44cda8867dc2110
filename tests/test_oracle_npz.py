"""The restated record layout of save_npz / load_npz (io.rs:49-316), on the CPU.

The reference's io tests (io.rs:350-436) round-trip an identity matrix and a
random matrix; the restatement must round-trip the same way, and its bytes
must follow the layout io.rs writes field by field.
"""
import struct

import numpy as np

from oracle import npz_format as N


def test_identity_round_trip():
    # io.rs:350-374: eye_array::<f64>(5, "csr")
    rec = N.record("csr_array", (5, 5), np.ones(5), np.arange(5), np.arange(6))
    fmt, shape, data, indices, indptr = N.parse(rec)
    assert fmt == "csr_array" and shape == (5, 5)
    assert list(data) == [1.0] * 5 and list(indices) == list(range(5)) and list(indptr) == list(range(6))


def test_layout_bytes():
    rec = N.record("csr_array", (2, 3), [1.5, -2.0], [0, 2], [0, 1, 2])
    expect = (struct.pack("<Q", 9) + b"csr_array" + struct.pack("<QQ", 2, 3)
              + struct.pack("<Q", 2) + struct.pack("<dd", 1.5, -2.0)
              + struct.pack("<Q", 2) + struct.pack("<QQ", 0, 2)
              + struct.pack("<Q", 3) + struct.pack("<QQQ", 0, 1, 2))
    assert rec == expect
    rec32 = N.record("csr_array", (2, 3), [1.5, -2.0], [0, 2], [0, 1, 2], dtype=np.float32)
    assert len(rec32) == len(rec) - 8


def test_random_round_trip_keeps_sum():
    # io.rs:402-436: nnz and the sum survive the round trip
    rng = np.random.default_rng(42)
    d = rng.uniform(size=30)
    rec = N.record("csr_array", (10, 10), d, rng.integers(0, 10, 30), np.linspace(0, 30, 11).astype(int))
    _, _, data, _, _ = N.parse(rec)
    assert len(data) == 30 and abs(data.sum() - d.sum()) < 1e-10
