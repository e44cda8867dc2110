"""Python host mirror of the scirs2-sparse iterative-solve API over the C ABI.

Names and argument meanings follow the reference crate (scirs2-sparse):
``CsrMatrix::new`` / ``CsrArray::from_triplets`` construction, the
``LinearOperator`` slot (operators and preconditioners are the same handle
type), and ``cg`` / ``bicgstab`` / ``gmres`` with their option defaults
(linalg/iterative.rs:17-35, :348-368, :614-634).  Errors surface as
``SparseError`` carrying the SparseError variant name, payload and Display
text (error.rs:9-74).  Every numeric operation runs in the CUDA library;
nothing here computes on the host.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L

_VARIANTS = {
    1: "ComputationError",
    2: "DimensionMismatch",
    3: "IndexOutOfBounds",
    4: "InvalidAxis",
    5: "InvalidSliceRange",
    6: "InconsistentData",
    7: "NotImplemented",
    8: "SingularMatrix",
    9: "ValueError",
    10: "ConversionError",
    11: "OperationNotSupported",
    12: "ShapeMismatch",
    13: "IterativeSolverFailure",
    14: "IndexCastOverflow",
    100: "CudaError",
    101: "DeviceTimeout",
    102: "InvalidArgument",
    103: "OutOfMemory",
}


class SparseError(Exception):
    """A non-zero status of the C ABI, with the SparseError payload."""

    def __init__(self, code: int, message: str, payload: tuple):
        super().__init__(message)
        self.code = code
        self.variant = _VARIANTS.get(code, "Unknown")
        self.payload = payload
        self.message = message


def _check(rc: int) -> None:
    if rc != 0:
        info = L.ErrorInfo()
        L.lib.sx_last_error(C.byref(info))
        raise SparseError(rc, info.message.decode("utf-8", "replace"),
                          (info.v0, info.v1, info.v2, info.v3))


def message_string(code: int) -> str:
    return L.lib.sx_message_string(code).decode("utf-8")


def mem_cache_trim() -> None:
    """Return the device blocks the library holds for reuse to the driver."""
    _check(L.lib.sx_mem_cache_trim())


def mem_cache_bytes() -> int:
    """Device bytes the library holds for reuse (freed blocks)."""
    return int(L.lib.sx_mem_cache_bytes())


_NP = {L.SX_F32: np.float32, L.SX_F64: np.float64}


def _dtype_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.float64:
        return L.SX_F64
    if dt == np.float32:
        return L.SX_F32
    raise TypeError(f"unsupported value type {dt}")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a.size else 0


class Context:
    """One CUDA stream, scratch and graph caches on one device."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        h = L.ctx_t()
        if stream is None:
            _check(L.lib.sx_ctx_create(device, C.byref(h)))
        else:
            _check(L.lib.sx_ctx_create_on_stream(device, C.c_void_p(stream), C.byref(h)))
        self.handle = h
        self.device = device

    @property
    def stream(self) -> int:
        return L.lib.sx_ctx_stream(self.handle) or 0

    @property
    def kernel_launches(self) -> int:
        return int(L.lib.sx_ctx_kernel_launches(self.handle))

    def synchronize(self) -> None:
        _check(L.lib.sx_ctx_synchronize(self.handle))

    def set_wait_limit(self, ns: int) -> None:
        """Limit of one dependency wait of the triangular factorisations and
        sweeps, in nanoseconds (0: the default of 2 s)."""
        _check(L.lib.sx_ctx_set_wait_limit(self.handle, int(ns)))

    def set_cg_recurrence(self, on: bool) -> None:
        """CG with a diagonal preconditioner in two kernels per iteration: A p
        carried by the recurrence q = A z + beta q (rounding differs slightly
        from the reference's loop).  Off by default."""
        _check(L.lib.sx_ctx_set_cg_recurrence(self.handle, 1 if on else 0))

    def wait_selftest(self):
        """One bounded device wait on a flag nothing sets: (gave_up, waited_ns).
        gave_up is True when the wait ran out at this context's limit."""
        w = C.c_uint64()
        rc = L.lib.sx_wait_selftest(self.handle, C.byref(w))
        if rc not in (0, 101):
            _check(rc)
        return rc == 101, int(w.value)

    def close(self) -> None:
        if self.handle:
            L.lib.sx_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Operator:
    """A device operator: CSR matrix, identity/diagonal operator or preconditioner."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle
        k = C.c_int()
        _check(L.lib.sx_op_kind_of(handle, C.byref(k)))
        self.kind = k.value
        d = C.c_int()
        _check(L.lib.sx_op_dtype(handle, C.byref(d)))
        self.dtype_code = d.value
        r, c = C.c_uint64(), C.c_uint64()
        _check(L.lib.sx_op_shape(handle, C.byref(r), C.byref(c)))
        self.shape = (r.value, c.value)
        self._keep = None

    @property
    def dtype(self):
        return _NP[self.dtype_code]

    def close(self) -> None:
        if self.handle:
            L.lib.sx_op_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # LinearOperator::matvec / rmatvec
    def matvec(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.empty(self.shape[0], dtype=self.dtype)
        _check(L.lib.sx_op_matvec(self.ctx.handle, self.handle, _ptr(x), x.size, _ptr(y), L.SX_MEM_HOST))
        return y

    @property
    def has_adjoint(self) -> bool:
        out = C.c_int()
        _check(L.lib.sx_op_has_adjoint(self.handle, C.byref(out)))
        return bool(out.value)

    def rmatvec(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.empty(self.shape[1], dtype=self.dtype)
        _check(L.lib.sx_op_rmatvec(self.ctx.handle, self.handle, _ptr(x), x.size, _ptr(y), L.SX_MEM_HOST))
        return y

    # CSR accessors
    def csr_info(self):
        r, c, n, s = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_int()
        _check(L.lib.sx_csr_info(self.handle, C.byref(r), C.byref(c), C.byref(n), C.byref(s)))
        return r.value, c.value, n.value, bool(s.value)

    @property
    def nnz(self) -> int:
        return self.csr_info()[2]

    @property
    def has_sorted_indices(self) -> bool:
        return self.csr_info()[3]

    def to_arrays(self):
        """(indptr, indices, data) as usize-like uint64 arrays and values."""
        nr, _, nnz, _ = self.csr_info()
        indptr = np.empty(nr + 1, dtype=np.uint64)
        indices = np.empty(nnz, dtype=np.uint64)
        data = np.empty(nnz, dtype=self.dtype)
        _check(L.lib.sx_csr_download(self.ctx.handle, self.handle, _ptr(indptr), _ptr(indices), _ptr(data)))
        return indptr, indices, data

    def get(self, i: int, j: int):
        out = np.zeros(1, dtype=self.dtype)
        _check(L.lib.sx_csr_get(self.ctx.handle, self.handle, i, j, _ptr(out)))
        return out[0]

    def transpose(self) -> "Operator":
        h = L.op_t()
        _check(L.lib.sx_csr_transpose(self.ctx.handle, self.handle, C.byref(h)))
        return Operator(self.ctx, h)

    def astype(self, dtype) -> "Operator":
        h = L.op_t()
        _check(L.lib.sx_csr_astype(self.ctx.handle, self.handle, _dtype_code(dtype), C.byref(h)))
        return Operator(self.ctx, h)

    def to_dense(self) -> np.ndarray:
        indptr, indices, data = self.to_arrays()
        d = np.zeros(self.shape, dtype=self.dtype)
        for r in range(self.shape[0]):
            for k in range(int(indptr[r]), int(indptr[r + 1])):
                d[r, int(indices[k])] = data[k]
        return d



class SymCsrMatrix(Operator):
    """SymCsrMatrix (sym_csr.rs:24-337): the lower triangle is stored, the
    operator applies the full symmetric matrix."""

    def nnz_stored(self) -> int:
        """SymCsrMatrix::nnz_stored (sym_csr.rs:241-243)."""
        a, _ = self._info()
        return a

    @property
    def nnz(self) -> int:
        """SymCsrMatrix::nnz (sym_csr.rs:254-268)."""
        _, b = self._info()
        return b

    def _info(self):
        a, b = C.c_uint64(), C.c_uint64()
        _check(L.lib.sx_sym_csr_info(self.ctx.handle, self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def to_arrays(self):
        """The stored (indptr, indices, data): the public fields of sym_csr.rs:28-34."""
        n = self.shape[0]
        nnz = self.nnz_stored()
        indptr = np.empty(n + 1, dtype=np.uint64)
        indices = np.empty(nnz, dtype=np.uint64)
        data = np.empty(nnz, dtype=self.dtype)
        _check(L.lib.sx_sym_csr_download(self.ctx.handle, self.handle, _ptr(indptr), _ptr(indices), _ptr(data)))
        return indptr, indices, data

    def to_csr(self) -> Operator:
        """SymCsrMatrix::to_csr (sym_csr.rs:305-337)."""
        h = L.op_t()
        _check(L.lib.sx_sym_csr_to_csr(self.ctx.handle, self.handle, C.byref(h)))
        return Operator(self.ctx, h)

    def to_dense(self) -> np.ndarray:
        """SymCsrMatrix::to_dense (sym_csr.rs:344-366): stored entries (the last
        duplicate wins), then the upper triangle mirrored from the lower."""
        indptr, indices, data = self.to_arrays()
        n = self.shape[0]
        d = np.zeros((n, n), dtype=self.dtype)
        for i in range(n):
            for k in range(int(indptr[i]), int(indptr[i + 1])):
                d[i, int(indices[k])] = data[k]
        for i in range(n):
            for j in range(i):
                d[j, i] = d[i, j]
        return d

    def astype(self, dtype) -> "SymCsrMatrix":
        indptr, indices, data = self.to_arrays()
        return sym_csr_matrix(self.ctx, data.astype(dtype), indptr, indices, self.shape, dtype=dtype)


def sym_csr_matrix(ctx: Context, data, indptr, indices, shape, dtype=np.float64) -> SymCsrMatrix:
    """SymCsrMatrix::new(data, indptr, indices, shape) (sym_csr.rs:64-134)."""
    data = np.ascontiguousarray(data, dtype=dtype)
    indptr = np.ascontiguousarray(indptr, dtype=np.uint64)
    indices = np.ascontiguousarray(indices, dtype=np.uint64)
    h = L.op_t()
    _check(L.lib.sx_sym_csr_new(ctx.handle, _dtype_code(dtype), _ptr(data), len(data), _ptr(indptr),
                                len(indptr), _ptr(indices), len(indices), int(shape[0]), int(shape[1]),
                                C.byref(h)))
    return SymCsrMatrix(ctx, h)


def sym_csr_from_csr(a: Operator) -> SymCsrMatrix:
    """SymCsrMatrix::from_csr(matrix) (sym_csr.rs:149-189)."""
    h = L.op_t()
    _check(L.lib.sx_sym_csr_from_csr(a.ctx.handle, a.handle, C.byref(h)))
    return SymCsrMatrix(a.ctx, h)


def sym_csr_matvec(a: SymCsrMatrix, x) -> np.ndarray:
    """sym_csr_matvec(matrix, x) (sym_ops.rs:56-90), bit for bit."""
    return a.matvec(x)


def sym_csr_quadratic_form(a: SymCsrMatrix, x):
    """sym_csr_quadratic_form(matrix, x) (sym_ops.rs:271-283), bit for bit."""
    x = np.ascontiguousarray(x, dtype=a.dtype)
    out = np.zeros(1, dtype=a.dtype)
    _check(L.lib.sx_sym_csr_quadratic_form(a.ctx.handle, a.handle, _ptr(x), x.size, L.SX_MEM_HOST, _ptr(out)))
    return out[0]


def sym_csr_trace(a: SymCsrMatrix):
    """sym_csr_trace(matrix) (sym_ops.rs:317-335), bit for bit."""
    out = np.zeros(1, dtype=a.dtype)
    _check(L.lib.sx_sym_csr_trace(a.ctx.handle, a.handle, _ptr(out)))
    return out[0]


def sym_csr_rank1_update(a: SymCsrMatrix, x, alpha) -> None:
    """sym_csr_rank1_update(matrix, x, alpha) (sym_ops.rs:179-233), in place."""
    x = np.ascontiguousarray(x, dtype=a.dtype)
    _check(L.lib.sx_sym_csr_rank1_update(a.ctx.handle, a.handle, _ptr(x), x.size, float(alpha), L.SX_MEM_HOST))

# ------------------------------------------------------------ construction
def csr_matrix(ctx: Context, data, rows, cols, shape, dtype=np.float64) -> Operator:
    """CsrMatrix::new(data, rows, cols, shape) (csr.rs:92-160)."""
    return _from_triplets(ctx, rows, cols, data, shape, dtype, L.SX_API_CSR_MATRIX, False)


def csr_array_from_triplets(ctx: Context, rows, cols, data, shape, sorted=False,
                            dtype=np.float64) -> Operator:
    """CsrArray::from_triplets(rows, cols, data, shape, sorted) (csr_array.rs:152-219)."""
    return _from_triplets(ctx, rows, cols, data, shape, dtype, L.SX_API_CSR_ARRAY, sorted)


def _from_triplets(ctx, rows, cols, data, shape, dtype, api, sorted_):
    data = np.ascontiguousarray(data, dtype=dtype)
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    cols = np.ascontiguousarray(cols, dtype=np.uint64)
    if not (len(rows) == len(cols) == len(data)):
        if api == L.SX_API_CSR_MATRIX:
            found = min(len(rows), len(cols))
            raise SparseError(2, f"Dimension mismatch: expected {len(data)}, found {found}",
                              (len(data), found, 0, 0))
        raise SparseError(6, "Inconsistent data: rows, cols, and data must have the same length",
                          (0, 0, 0, 0))
    h = L.op_t()
    _check(L.lib.sx_csr_from_triplets(ctx.handle, _dtype_code(dtype), api, _ptr(rows), _ptr(cols),
                                      _ptr(data), len(data), int(shape[0]), int(shape[1]),
                                      1 if sorted_ else 0, C.byref(h)))
    return Operator(ctx, h)


def csr_matrix_from_raw(ctx: Context, data, indptr, indices, shape, dtype=np.float64) -> Operator:
    """CsrMatrix::from_raw_csr(data, indptr, indices, shape) (csr.rs:174-227)."""
    return _from_raw(ctx, data, indptr, indices, shape, dtype, L.SX_API_CSR_MATRIX)


def csr_array(ctx: Context, data, indices, indptr, shape, dtype=np.float64) -> Operator:
    """CsrArray::new(data, indices, indptr, shape) (csr_array.rs:77-136)."""
    return _from_raw(ctx, data, indptr, indices, shape, dtype, L.SX_API_CSR_ARRAY)


def _from_raw(ctx, data, indptr, indices, shape, dtype, api):
    data = np.ascontiguousarray(data, dtype=dtype)
    indptr = np.ascontiguousarray(indptr, dtype=np.uint64)
    indices = np.ascontiguousarray(indices, dtype=np.uint64)
    if len(data) != len(indices):
        if api == L.SX_API_CSR_MATRIX:
            raise SparseError(2, f"Dimension mismatch: expected {len(data)}, found {len(indices)}",
                              (len(data), len(indices), 0, 0))
        raise SparseError(6, "Inconsistent data: data and indices must have the same length",
                          (0, 0, 0, 0))
    h = L.op_t()
    _check(L.lib.sx_csr_from_raw(ctx.handle, _dtype_code(dtype), api, _ptr(indptr), len(indptr),
                                 _ptr(indices), _ptr(data), len(data), int(shape[0]), int(shape[1]),
                                 C.byref(h)))
    return Operator(ctx, h)


def save_npz(a: Operator, path) -> None:
    """save_npz(&array, path) (io.rs:49-177): the reference's "csr_array" record."""
    _check(L.lib.sx_csr_save_npz(a.ctx.handle, a.handle, os.fsencode(path)))


def load_npz(ctx: Context, path, dtype=np.float64) -> Operator:
    """load_npz::<T, _>(path) (io.rs:197-269) of a "csr_array" record, onto the device."""
    h = L.op_t()
    _check(L.lib.sx_csr_load_npz(ctx.handle, _dtype_code(dtype), os.fsencode(path), C.byref(h)))
    return Operator(ctx, h)


def spmv_kernel(op: Operator, exact: bool = True, sym_half: bool = False) -> str:
    """Name of the SpMV kernel the library launches for `op` (diagnostics)."""
    buf = C.create_string_buffer(256)
    flags = (L.SX_SPMV_EXACT if exact else 0) | (L.SX_SPMV_SYM_HALF if sym_half else 0)
    _check(L.lib.sx_spmv_kernel(op.ctx.handle, op.handle, flags, buf, 256))
    return buf.value.decode()


def csr_from_arrays(ctx: Context, indptr, indices, data, shape, dtype=None) -> Operator:
    """Device-native upload of int64 row pointers / int32 columns (host numpy)."""
    dtype = dtype or np.asarray(data).dtype
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=dtype)
    h = L.op_t()
    _check(L.lib.sx_csr_from_raw_i32(ctx.handle, _dtype_code(dtype), _ptr(indptr), _ptr(indices),
                                     _ptr(data), int(shape[0]), int(shape[1]), len(data),
                                     L.SX_MEM_HOST, C.byref(h)))
    return Operator(ctx, h)


def identity(ctx: Context, n: int, dtype=np.float64) -> Operator:
    h = L.op_t()
    _check(L.lib.sx_op_identity(ctx.handle, _dtype_code(dtype), n, C.byref(h)))
    return Operator(ctx, h)


def scaled_identity(ctx: Context, n: int, scale: float, dtype=np.float64) -> Operator:
    h = L.op_t()
    _check(L.lib.sx_op_scaled_identity(ctx.handle, _dtype_code(dtype), n, float(scale), C.byref(h)))
    return Operator(ctx, h)


def diagonal(ctx: Context, diag, dtype=np.float64) -> Operator:
    d = np.ascontiguousarray(diag, dtype=dtype)
    h = L.op_t()
    _check(L.lib.sx_op_diagonal(ctx.handle, _dtype_code(dtype), _ptr(d), d.size, C.byref(h)))
    return Operator(ctx, h)


def zero_operator(ctx: Context, nrows: int, ncols: int, dtype=np.float64) -> Operator:
    """ZeroOperator::new(rows, cols) (interface.rs:184-191)."""
    h = L.op_t()
    _check(L.lib.sx_op_zero(ctx.handle, _dtype_code(dtype), nrows, ncols, C.byref(h)))
    return Operator(ctx, h)


def sum_operator(a: Operator, b: Operator) -> Operator:
    """SumOperator::new(a, b) (interface.rs:306-316).  The result borrows a
    and b: keep them open while it is used."""
    h = L.op_t()
    _check(L.lib.sx_op_sum(a.ctx.handle, a.handle, b.handle, C.byref(h)))
    op = Operator(a.ctx, h)
    op._operands = (a, b)
    return op


def product_operator(a: Operator, b: Operator) -> Operator:
    """ProductOperator::new(a, b): (A B) x = A (B x) (interface.rs:358-370).
    The result borrows a and b."""
    h = L.op_t()
    _check(L.lib.sx_op_product(a.ctx.handle, a.handle, b.handle, C.byref(h)))
    op = Operator(a.ctx, h)
    op._operands = (a, b)
    return op


def host_operator(ctx: Context, n: int, fn, dtype=np.float64) -> Operator:
    """A user LinearOperator whose matvec runs in Python (staged copies)."""
    npdt = np.dtype(dtype)

    def cb(user, x, y, nn):
        xs = np.ctypeslib.as_array(C.cast(x, C.POINTER(C.c_double if npdt == np.float64 else C.c_float)), (nn,))
        ys = np.ctypeslib.as_array(C.cast(y, C.POINTER(C.c_double if npdt == np.float64 else C.c_float)), (n,))
        ys[:] = fn(xs.copy())
        return 0

    cfn = L.HOST_MATVEC_FN(cb)
    h = L.op_t()
    _check(L.lib.sx_op_host(ctx.handle, _dtype_code(dtype), n, n, cfn, None, C.byref(h)))
    op = Operator(ctx, h)
    op._keep = cfn
    return op


def jacobi(ctx: Context, a: Operator) -> Operator:
    """JacobiPreconditioner::new(&matrix) (preconditioners.rs:21-44)."""
    h = L.op_t()
    _check(L.lib.sx_precond_jacobi(ctx.handle, a.handle, C.byref(h)))
    return Operator(ctx, h)


def jacobi_from_diagonal(ctx: Context, diag, dtype=np.float64) -> Operator:
    """JacobiPreconditioner::from_diagonal (preconditioners.rs:47-62)."""
    d = np.ascontiguousarray(diag, dtype=dtype)
    h = L.op_t()
    _check(L.lib.sx_precond_jacobi_from_diagonal(ctx.handle, _dtype_code(dtype), _ptr(d), d.size, C.byref(h)))
    return Operator(ctx, h)


def ic0(ctx: Context, a: Operator, textbook: bool = False) -> Operator:
    """IC0Preconditioner::new(&matrix) (ic.rs:22-135); textbook=True gives standard IC(0)."""
    h = L.op_t()
    _check(L.lib.sx_precond_ic0(ctx.handle, a.handle,
                                L.SX_IC0_TEXTBOOK if textbook else L.SX_IC0_REFERENCE, C.byref(h)))
    return Operator(ctx, h)


def ilu0(ctx: Context, a: Operator) -> Operator:
    """ILU0Preconditioner::new(&matrix) (preconditioners.rs:209-324)."""
    h = L.op_t()
    _check(L.lib.sx_precond_ilu0(ctx.handle, a.handle, C.byref(h)))
    return Operator(ctx, h)


def ssor(ctx: Context, a: Operator, omega: float) -> Operator:
    """SSORPreconditioner::new(matrix, omega) (preconditioners.rs:103-131)."""
    h = L.op_t()
    _check(L.lib.sx_precond_ssor(ctx.handle, a.handle, float(omega), C.byref(h)))
    return Operator(ctx, h)


def fsai(ctx: Context, g: Operator) -> Operator:
    """M^-1 = G G^T from a lower-triangular CSR G."""
    h = L.op_t()
    _check(L.lib.sx_precond_fsai(ctx.handle, g.handle, C.byref(h)))
    return Operator(ctx, h)


# ----------------------------------------------------------------- solvers
@dataclass
class IterationResult:
    """IterationResult (iterative.rs:8-14)."""
    x: np.ndarray
    iterations: int
    residual_norm: float
    converged: bool
    message: str


def _result(x, r: L.IterResult) -> IterationResult:
    buf = C.create_string_buffer(512)
    _check(L.lib.sx_iter_message(C.byref(r), L.SX_F64 if x.dtype == np.float64 else L.SX_F32, buf, 512))
    return IterationResult(x, int(r.iterations), float(r.residual_norm), bool(r.converged),
                           buf.value.decode("utf-8"))


def _prep(a: Operator, b, x0):
    b = np.ascontiguousarray(b, dtype=a.dtype)
    x = np.empty(a.shape[0], dtype=a.dtype)
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=a.dtype)
    if x0a is not None and x0a.size != a.shape[0]:
        raise SparseError(2, f"Dimension mismatch: expected {a.shape[0]}, found {x0a.size}",
                          (a.shape[0], x0a.size, 0, 0))
    return b, x, x0a


def cg(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
       preconditioner: Optional[Operator] = None) -> IterationResult:
    """cg(a, b, CGOptions { .. }) (iterative.rs:40-162)."""
    b, x, x0a = _prep(a, b, x0)
    o = L.CGOptions(max_iter, rtol, atol, _ptr(x0a) if x0a is not None else None,
                    preconditioner.handle if preconditioner else None)
    r = L.IterResult()
    _check(L.lib.sx_cg(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST, C.byref(r)))
    return _result(x, r)


def bicgstab(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
             left_preconditioner: Optional[Operator] = None,
             right_preconditioner: Optional[Operator] = None) -> IterationResult:
    """bicgstab(a, b, BiCGSTABOptions { .. }) (iterative.rs:377-611)."""
    b, x, x0a = _prep(a, b, x0)
    o = L.BiCGSTABOptions(max_iter, rtol, atol, _ptr(x0a) if x0a is not None else None,
                          left_preconditioner.handle if left_preconditioner else None,
                          right_preconditioner.handle if right_preconditioner else None)
    r = L.IterResult()
    _check(L.lib.sx_bicgstab(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST, C.byref(r)))
    return _result(x, r)


def gmres(a: Operator, b, max_iter=1000, restart=30, rtol=1e-8, atol=1e-12, x0=None,
          preconditioner: Optional[Operator] = None) -> IterationResult:
    """gmres(a, b, GMRESOptions { .. }) (iterative.rs:641-816)."""
    b, x, x0a = _prep(a, b, x0)
    o = L.GMRESOptions(max_iter, restart, rtol, atol, _ptr(x0a) if x0a is not None else None,
                       preconditioner.handle if preconditioner else None)
    r = L.IterResult()
    _check(L.lib.sx_gmres(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST, C.byref(r)))
    return _result(x, r)


def _bicg_like(fn, a: Operator, b, max_iter, rtol, atol, x0, left, right) -> IterationResult:
    b, x, x0a = _prep(a, b, x0)
    o = L.BiCGOptions(max_iter, rtol, atol, _ptr(x0a) if x0a is not None else None,
                      left.handle if left else None, right.handle if right else None)
    r = L.IterResult()
    _check(fn(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST, C.byref(r)))
    return _result(x, r)


def bicg(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
         left_preconditioner: Optional[Operator] = None,
         right_preconditioner: Optional[Operator] = None) -> IterationResult:
    """bicg(a, b, BiCGOptions { .. }) (iterative.rs:189-345)."""
    return _bicg_like(L.lib.sx_bicg, a, b, max_iter, rtol, atol, x0, left_preconditioner, right_preconditioner)


def cgs(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
        left_preconditioner: Optional[Operator] = None,
        right_preconditioner: Optional[Operator] = None) -> IterationResult:
    """cgs(a, b, CGSOptions { .. }) (cgs.rs:15-193); the left preconditioner is unused."""
    return _bicg_like(L.lib.sx_cgs, a, b, max_iter, rtol, atol, x0, left_preconditioner, right_preconditioner)


def qmr(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
        left_preconditioner: Optional[Operator] = None,
        right_preconditioner: Optional[Operator] = None) -> IterationResult:
    """qmr(a, b, QMROptions { .. }) (qmr.rs:44-259)."""
    return _bicg_like(L.lib.sx_qmr, a, b, max_iter, rtol, atol, x0, left_preconditioner, right_preconditioner)


def minres(a: Operator, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None,
           preconditioner: Optional[Operator] = None) -> IterationResult:
    """minres(a, b, MINRESOptions { .. }) (minres.rs:66-257)."""
    b, x, x0a = _prep(a, b, x0)
    o = L.MINRESOptions(max_iter, rtol, atol, _ptr(x0a) if x0a is not None else None,
                        preconditioner.handle if preconditioner else None)
    r = L.IterResult()
    _check(L.lib.sx_minres(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST,
                           C.byref(r)))
    return _result(x, r)


def lgmres(a: Operator, b, max_iter=500, rtol=1e-8, atol=1e-8, inner_m=30, outer_k=3, x0=None,
           preconditioner: Optional[Operator] = None) -> IterationResult:
    """lgmres(a, b, LGMRESOptions { .. }) (lgmres.rs:58-327).  LGMRESResult has no
    message; the returned one is "Converged" or "Maximum iterations reached"."""
    b, x, x0a = _prep(a, b, x0)
    o = L.LGMRESOptions(max_iter, rtol, atol, inner_m, outer_k, _ptr(x0a) if x0a is not None else None,
                        preconditioner.handle if preconditioner else None)
    r = L.IterResult()
    _check(L.lib.sx_lgmres(a.ctx.handle, a.handle, _ptr(b), b.size, C.byref(o), _ptr(x), L.SX_MEM_HOST,
                           C.byref(r)))
    return _result(x, r)


# ----------------------------------------------------------- eigenpairs
@dataclass
class EigenResult:
    """EigenResult (eigen.rs:64-78): eigenvectors is n x k (column k = pair k)."""
    eigenvalues: np.ndarray
    eigenvectors: Optional[np.ndarray]
    iterations: int
    residuals: np.ndarray
    converged: bool


def power_iteration(a: SymCsrMatrix, max_iter=100, tol=1e-8, normalize=True, initial_guess=None) -> EigenResult:
    """power_iteration(matrix, PowerIterationOptions { .. }, initial_guess)
    (eigen.rs:124-293)."""
    n = a.shape[0]
    x0 = None if initial_guess is None else np.ascontiguousarray(initial_guess, dtype=a.dtype)
    o = L.PowerOptions(max_iter, tol, 1 if normalize else 0)
    lam = np.zeros(1, dtype=a.dtype)
    res = np.zeros(1, dtype=a.dtype)
    vec = np.zeros(n, dtype=a.dtype)
    r = L.EigenResult()
    _check(L.lib.sx_power_iteration(a.ctx.handle, a.handle, C.byref(o), _ptr(x0) if x0 is not None else None,
                                    0 if x0 is None else x0.size, L.SX_MEM_HOST, _ptr(lam), _ptr(vec), _ptr(res),
                                    C.byref(r)))
    return EigenResult(lam, vec.reshape(n, 1), int(r.iterations), res, bool(r.converged))


def lanczos(a: SymCsrMatrix, max_iter=1000, max_subspace_size=20, tol=1e-8, num_eigenvalues=1,
            compute_eigenvectors=True, initial_guess=None) -> EigenResult:
    """lanczos(matrix, LanczosOptions { .. }, initial_guess) (eigen.rs:295-494)."""
    n = a.shape[0]
    x0 = None if initial_guess is None else np.ascontiguousarray(initial_guess, dtype=a.dtype)
    o = L.LanczosOptions(max_iter, max_subspace_size, tol, num_eigenvalues, 1 if compute_eigenvectors else 0)
    k = max(min(num_eigenvalues, max_subspace_size, n), 1)
    vals = np.zeros(k, dtype=a.dtype)
    res = np.zeros(k, dtype=a.dtype)
    vecs = np.zeros(n * k, dtype=a.dtype) if compute_eigenvectors else None
    r = L.EigenResult()
    _check(L.lib.sx_lanczos(a.ctx.handle, a.handle, C.byref(o), _ptr(x0) if x0 is not None else None,
                            0 if x0 is None else x0.size, L.SX_MEM_HOST, _ptr(vals),
                            _ptr(vecs) if vecs is not None else None, _ptr(res), C.byref(r)))
    cols = int(r.num_columns)
    ev = vecs[: n * cols].reshape(n, cols) if vecs is not None else None
    return EigenResult(vals[: int(r.num_eigenvalues)], ev, int(r.iterations), res[:cols], bool(r.converged))


@dataclass
class IRResult:
    x: np.ndarray
    outer_iterations: int
    inner_iterations: int
    rel_residual: float
    converged: bool


def cg_mixed(a64: Operator, b, tol=1e-10, inner_rtol=1e-4, max_outer=30, max_inner=10000,
             x0=None, preconditioner: Optional[Operator] = None,
             a32: Optional[Operator] = None, mode: str = "replace",
             replace_factor: float = 0.1) -> IRResult:
    """FP32 PCG inside an FP64 refinement loop (no reference counterpart).

    mode "replace": one FP32 CG run whose residual is replaced by the FP64
    true residual each time it has fallen by `replace_factor`; mode
    "restart": classic refinement, a fresh FP32 PCG to `inner_rtol` per
    correction."""
    if mode not in ("replace", "restart"):
        raise ValueError("mode must be 'replace' or 'restart'")
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(a64.shape[0], dtype=np.float64)
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    o = L.IROptions()
    L.lib.sx_ir_options_default(C.byref(o))
    o.max_outer, o.max_inner, o.tol, o.inner_rtol = max_outer, max_inner, tol, inner_rtol
    o.x0 = _ptr(x0a) if x0a is not None else None
    o.preconditioner = preconditioner.handle if preconditioner else None
    o.a32 = a32.handle if a32 else None
    o.mode = L.SX_IR_REPLACE if mode == "replace" else L.SX_IR_RESTART
    o.replace_factor = replace_factor
    r = L.IRResult()
    _check(L.lib.sx_cg_mixed(a64.ctx.handle, a64.handle, _ptr(b), b.size, C.byref(o), _ptr(x),
                             L.SX_MEM_HOST, C.byref(r)))
    return IRResult(x, int(r.outer_iterations), int(r.inner_iterations), float(r.rel_residual),
                    bool(r.converged))


class LearnedSAI:
    """The message-passing network that predicts G for M^-1 = G G^T."""

    def __init__(self, ctx: Context, params=None, seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        pp = None
        if params is not None:
            params = np.ascontiguousarray(params, dtype=np.float32)
            pp = _ptr(params)
        _check(L.lib.sx_gnn_create(ctx.handle, pp, seed, C.byref(h)))
        self.handle = h
        self.num_params = int(L.lib.sx_gnn_num_params())

    def close(self):
        if self.handle:
            L.lib.sx_gnn_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        _check(L.lib.sx_gnn_get_params(self.ctx.handle, self.handle, _ptr(out)))
        return out

    @params.setter
    def params(self, value):
        value = np.ascontiguousarray(value, dtype=np.float32)
        _check(L.lib.sx_gnn_set_params(self.ctx.handle, self.handle, _ptr(value)))

    def loss_grad(self, a: Operator, probes=None, seed: int = 0):
        grad = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_float()
        pp = None
        if probes is not None:
            probes = np.ascontiguousarray(probes, dtype=np.float32)
            pp = _ptr(probes)
        _check(L.lib.sx_gnn_loss_grad(self.ctx.handle, self.handle, a.handle, pp, seed, C.byref(loss),
                                      _ptr(grad)))
        return float(loss.value), grad

    def train_step(self, a: Operator, seed: int, lr: float = 1e-3) -> float:
        loss = C.c_float()
        _check(L.lib.sx_gnn_train_step(self.ctx.handle, self.handle, a.handle, seed, lr, C.byref(loss)))
        return float(loss.value)

    def edge_values(self, a: Operator) -> np.ndarray:
        ng = C.c_uint64()
        _check(L.lib.sx_gnn_edge_values(self.ctx.handle, self.handle, a.handle, None, C.byref(ng)))
        out = np.empty(ng.value, dtype=np.float32)
        _check(L.lib.sx_gnn_edge_values(self.ctx.handle, self.handle, a.handle, _ptr(out), C.byref(ng)))
        return out

    def preconditioner(self, a: Operator) -> Operator:
        h = L.op_t()
        _check(L.lib.sx_precond_learned(self.ctx.handle, a.handle, self.handle, C.byref(h)))
        return Operator(self.ctx, h)


@dataclass
class BatchedResult:
    x: np.ndarray
    inner_iterations: np.ndarray
    rel_residual: np.ndarray
    converged: np.ndarray
    outer_iterations: int
    kernel_launches: int
    threads_per_block: int = 0  # launch shape the autotuner chose
    blocks_per_sm: int = 0


def batched_pcg(a64: Operator, sys_ptr, b, rtol=1e-8, atol=0.0, inner_rtol=1e-4, max_iter=10000,
                max_outer=30, a32: Optional[Operator] = None) -> BatchedResult:
    """Batched FP64-refined FP32 Jacobi-PCG over a block-diagonal CSR."""
    sys_ptr = np.ascontiguousarray(sys_ptr, dtype=np.int64)
    nsys = len(sys_ptr) - 1
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(a64.shape[0], dtype=np.float64)
    o = L.BatchedOptions(max_iter, rtol, atol, inner_rtol, max_outer)
    per = (L.BatchedResult * max(nsys, 1))()
    summ = L.BatchedSummary()
    _check(L.lib.sx_batched_pcg(a64.ctx.handle, a64.handle, a32.handle if a32 else None, _ptr(sys_ptr),
                                nsys, _ptr(b), _ptr(x), C.byref(o), L.SX_MEM_HOST, per, C.byref(summ)))
    return BatchedResult(x,
                         np.array([per[i].inner_iterations for i in range(nsys)], dtype=np.int64),
                         np.array([per[i].rel_residual for i in range(nsys)]),
                         np.array([bool(per[i].converged) for i in range(nsys)]),
                         int(summ.outer_iterations), int(summ.kernel_launches),
                         int(summ.threads_per_block), int(summ.blocks_per_sm))


def generate_batch(nsys: int, side_min: int, side_max: int, seed: int = 0, sigma: float = 1.0):
    """Block-diagonal batch of 2D variable-coefficient systems:
    (sys_ptr, indptr, indices, values)."""
    sys_ptr = np.empty(nsys + 1, dtype=np.int64)
    n, nnz = C.c_int64(), C.c_int64()
    rc = L.lib.sx_gen_batch_varcoef2d(nsys, side_min, side_max, seed, sigma, _ptr(sys_ptr), C.byref(n),
                                      C.byref(nnz), None, None, None)
    if rc:
        raise ValueError(f"batch generator failed ({rc})")
    indptr = np.empty(n.value + 1, dtype=np.int64)
    indices = np.empty(nnz.value, dtype=np.int32)
    vals = np.empty(nnz.value, dtype=np.float64)
    rc = L.lib.sx_gen_batch_varcoef2d(nsys, side_min, side_max, seed, sigma, _ptr(sys_ptr), C.byref(n),
                                      C.byref(nnz), _ptr(indptr), _ptr(indices), _ptr(vals))
    if rc:
        raise ValueError(f"batch generator failed ({rc})")
    return sys_ptr, indptr, indices, vals


def true_rel_residual(a64: Operator, b, x) -> float:
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = C.c_double()
    _check(L.lib.sx_true_rel_residual(a64.ctx.handle, a64.handle, _ptr(b), _ptr(x), L.SX_MEM_HOST,
                                      C.byref(out)))
    return out.value


# -------------------------------------------------------------- generators
GEN_KINDS = {"poisson2d": 0, "laplace3d": 1, "varcoef3d": 2, "varcoef2d": 3, "aniso_q1": 4,
             "powerlaw": 5}


def generate(kind: str, nx: int, ny: int = 1, nz: int = 1, seed: int = 0, param0: float = 0.0,
             param1: float = 0.0):
    """Seeded synthetic CSR: returns (indptr int64, indices int32, values float64)."""
    spec = L.GenSpec(GEN_KINDS[kind], nx, ny, nz, seed, param0, param1)
    n, nnz = C.c_int64(), C.c_int64()
    rc = L.lib.sx_gen_matrix(C.byref(spec), C.byref(n), C.byref(nnz), None, None, None)
    if rc:
        raise ValueError(f"generator {kind} rejected its arguments ({rc})")
    indptr = np.empty(n.value + 1, dtype=np.int64)
    indices = np.empty(nnz.value, dtype=np.int32)
    vals = np.empty(nnz.value, dtype=np.float64)
    rc = L.lib.sx_gen_matrix(C.byref(spec), C.byref(n), C.byref(nnz), _ptr(indptr), _ptr(indices), _ptr(vals))
    if rc:
        raise ValueError(f"generator {kind} failed ({rc})")
    return indptr, indices, vals


def rhs_normal(seed: int, n: int) -> np.ndarray:
    b = np.empty(n, dtype=np.float64)
    L.lib.sx_gen_rhs_normal(seed, n, _ptr(b))
    return b
