"""The reference's sparse-array record (scirs2-sparse src/io.rs:49-316), restated.

TEST INFRASTRUCTURE ONLY: tests/ use it to write the files the reference would
write and to read files back in its layout; the library never imports it.

Layout (little-endian): write_string(format) = u64 length + bytes;
write_usize(rows), write_usize(cols); write_array(data) = u64 length + the
values' bytes; write_array(indices) (u64 each); then write_array(indptr) for
CSR / CSC records or write_array(cols) for COO / DOK records.
"""
import struct

import numpy as np


def _array(values, dtype):
    a = np.ascontiguousarray(values, dtype=dtype)
    return struct.pack("<Q", a.size) + a.astype(a.dtype.newbyteorder("<")).tobytes()


def record(fmt, shape, data, indices, last, dtype=np.float64):
    """Bytes of save_npz (io.rs:152-175) for the given record parts."""
    b = fmt.encode() if isinstance(fmt, str) else bytes(fmt)
    out = struct.pack("<Q", len(b)) + b
    out += struct.pack("<QQ", int(shape[0]), int(shape[1]))
    out += _array(data, dtype)
    out += _array(indices, np.uint64)
    out += _array(last, np.uint64)
    return out


def parse(buf, dtype=np.float64):
    """load_npz's reads (io.rs:212-233): (format, shape, data, indices, last)."""
    o = 0

    def take(n):
        nonlocal o
        if o + n > len(buf):
            raise EOFError("failed to fill whole buffer")
        v = buf[o:o + n]
        o += n
        return v

    (flen,) = struct.unpack("<Q", take(8))
    fmt = take(flen).decode("utf-8")
    rows, cols = struct.unpack("<QQ", take(16))
    w = np.dtype(dtype).itemsize

    def arr(dt, width):
        (n,) = struct.unpack("<Q", take(8))
        return np.frombuffer(take(n * width), dtype=np.dtype(dt).newbyteorder("<")).copy()

    data = arr(dtype, w)
    indices = arr(np.uint64, 8)
    last = arr(np.uint64, 8)
    return fmt, (rows, cols), data, indices, last
