"""ctypes loader of the CPU oracle (test infrastructure only).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker or the timed CPU baseline.  Builds the oracle with its
Makefile on first use.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsx_oracle.so")


def build() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


class Err(C.Structure):
    _fields_ = [("code", C.c_int), ("v0", C.c_uint64), ("v1", C.c_uint64), ("v2", C.c_uint64),
                ("v3", C.c_uint64), ("msg", C.c_char * 256)]


class Res(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("residual_norm", C.c_double), ("converged", C.c_int),
                ("message", C.c_int)]


class EigInfo(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("converged", C.c_int), ("count", C.c_uint64), ("num", C.c_uint64)]


class IROpt(C.Structure):
    _fields_ = [("max_outer", C.c_uint64), ("max_inner", C.c_uint64), ("tol", C.c_double),
                ("inner_rtol", C.c_double), ("jacobi", C.c_int)]


class IRRes(C.Structure):
    _fields_ = [("outer_iterations", C.c_uint64), ("inner_iterations", C.c_uint64),
                ("rel_residual", C.c_double), ("converged", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, u64, i64, dbl, ip = C.c_void_p, C.c_uint64, C.c_int64, C.c_double, C.c_int
        E = C.POINTER(Err)
        sig = {
            "or_csr_matrix_new_f64": (ip, [vp, vp, vp, u64, u64, u64, vp, vp, vp, E]),
            "or_csr_matrix_new_f32": (ip, [vp, vp, vp, u64, u64, u64, vp, vp, vp, E]),
            "or_csr_matrix_from_raw_check": (ip, [vp, u64, vp, u64, u64, u64, u64, E]),
            "or_csr_array_new_check": (ip, [vp, u64, vp, u64, u64, u64, u64, vp, E]),
            "or_csr_array_from_triplets_f64": (ip, [vp, vp, vp, u64, u64, u64, ip, vp, vp, vp, vp, E]),
            "or_csr_array_from_triplets_f32": (ip, [vp, vp, vp, u64, u64, u64, ip, vp, vp, vp, vp, E]),
            "or_csr_transpose_f64": (None, [vp, vp, vp, u64, u64, vp, vp, vp]),
            "or_csr_transpose_f32": (None, [vp, vp, vp, u64, u64, vp, vp, vp]),
            "or_csr_get_f64": (dbl, [vp, vp, vp, u64, u64, u64, u64]),
            "or_spmv_f64": (None, [vp, vp, vp, u64, vp, vp]),
            "or_spmv_f32": (None, [vp, vp, vp, u64, vp, vp]),
            "or_spmv_i32_f64": (None, [vp, vp, vp, i64, vp, vp]),
            "or_spmv_i32_f32": (None, [vp, vp, vp, i64, vp, vp]),
            "or_op_csr": (vp, [ip, vp, vp, vp, u64, u64]),
            "or_op_csr_i32": (vp, [ip, vp, vp, vp, i64, i64]),
            "or_op_identity": (vp, [ip, u64]),
            "or_op_scaled_identity": (vp, [ip, u64, dbl]),
            "or_op_diagonal": (vp, [ip, vp, u64]),
            "or_op_jacobi": (vp, [vp, E]),
            "or_op_jacobi_from_diagonal": (vp, [ip, vp, u64, E]),
            "or_op_ic0": (vp, [vp, ip, E]),
            "or_op_fsai": (vp, [vp]),
            "or_op_ilu0": (vp, [vp, E]),
            "or_op_ssor": (vp, [vp, dbl, E]),
            "or_op_destroy": (None, [vp]),
            "or_op_matvec": (ip, [vp, vp, vp]),
            "or_op_rows": (u64, [vp]),
            "or_ic0_nnz": (u64, [vp]),
            "or_ic0_factor": (None, [vp, vp, vp, vp]),
            "or_cg": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, C.POINTER(Res), E]),
            "or_bicgstab": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, vp, C.POINTER(Res), E]),
            "or_gmres": (ip, [vp, vp, u64, u64, dbl, dbl, vp, vp, vp, C.POINTER(Res), E]),
            "or_cg_mixed_ir": (ip, [vp, vp, vp, i64, vp, C.POINTER(IROpt), vp, C.POINTER(IRRes)]),
            "or_cg_mixed_replace": (ip, [vp, vp, vp, i64, vp, C.POINTER(IROpt), C.c_double, vp,
                                         C.POINTER(IRRes)]),
            "or_true_rel_residual": (dbl, [vp, vp, vp, i64, vp, vp]),
            "or_bicg": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, vp, C.POINTER(Res), E]),
            "or_cgs": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, C.POINTER(Res), E]),
            "or_qmr": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, vp, C.POINTER(Res), E]),
            "or_minres": (ip, [vp, vp, u64, dbl, dbl, vp, vp, vp, C.POINTER(Res), E]),
            "or_lgmres": (ip, [vp, vp, u64, u64, dbl, dbl, vp, vp, vp, C.POINTER(Res), E]),
            "or_sym_csr_check": (ip, [u64, vp, u64, vp, u64, u64, u64, E]),
            "or_sym_csr_matvec_f64": (None, [vp, vp, vp, u64, vp, vp]),
            "or_sym_csr_matvec_f32": (None, [vp, vp, vp, u64, vp, vp]),
            "or_sym_csr_nnz": (u64, [vp, vp, u64, u64]),
            "or_sym_csr_get_f64": (dbl, [vp, vp, vp, u64, u64, u64]),
            "or_sym_csr_trace_f64": (dbl, [vp, vp, vp, u64]),
            "or_sym_csr_trace_f32": (C.c_float, [vp, vp, vp, u64]),
            "or_sym_csr_quadratic_form_f64": (dbl, [vp, vp, vp, u64, vp]),
            "or_sym_csr_quadratic_form_f32": (C.c_float, [vp, vp, vp, u64, vp]),
            "or_sym_csr_rank1_update_f64": (u64, [vp, vp, vp, u64, vp, dbl, vp, vp, vp]),
            "or_sym_csr_rank1_update_f32": (u64, [vp, vp, vp, u64, vp, C.c_float, vp, vp, vp]),
            "or_sym_csr_from_csr_f64": (ip, [vp, vp, vp, u64, u64, vp, vp, vp, E]),
            "or_sym_csr_from_csr_f32": (ip, [vp, vp, vp, u64, u64, vp, vp, vp, E]),
            "or_power_iteration_f64": (ip, [vp, vp, vp, u64, u64, dbl, ip, vp, u64, vp, vp, vp,
                                            C.POINTER(EigInfo), E]),
            "or_power_iteration_f32": (ip, [vp, vp, vp, u64, u64, dbl, ip, vp, u64, vp, vp, vp,
                                            C.POINTER(EigInfo), E]),
            "or_lanczos_f64": (ip, [vp, vp, vp, u64, u64, u64, dbl, u64, ip, vp, u64, vp, vp, vp,
                                    C.POINTER(EigInfo), E]),
            "or_lanczos_f32": (ip, [vp, vp, vp, u64, u64, u64, dbl, u64, ip, vp, u64, vp, vp, vp,
                                    C.POINTER(EigInfo), E]),
            "or_tridiag_eig_f64": (ip, [vp, vp, u64, u64, u64, vp, vp, vp, E]),
            "or_solve_cubic_f64": (u64, [dbl, dbl, dbl, vp]),
            "or_set_threads": (None, [ip]),
            "or_get_threads": (ip, []),
            "or_gen_matrix": (ip, [ip, i64, i64, i64, u64, dbl, dbl, C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64), vp, vp, vp]),
            "or_gen_batch_sides": (None, [u64, i64, i64, u64, vp]),
            "or_gen_batch_system_seed": (u64, [u64, u64]),
            "or_gen_rhs_normal": (None, [u64, i64, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def p(a: np.ndarray):
    return a.ctypes.data if a is not None and a.size else None


class Op:
    """An oracle LinearOperator handle."""

    def __init__(self, handle, n, f64=True):
        self.h = handle
        self.n = n
        self.f64 = f64

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_op_destroy(self.h)
            self.h = None

    def matvec(self, x):
        dt = np.float64 if self.f64 else np.float32
        x = np.ascontiguousarray(x, dtype=dt)
        y = np.empty(self.n, dtype=dt)
        lib().or_op_matvec(self.h, p(x), p(y))
        return y


def op_csr(indptr, indices, data, shape):
    f64 = np.asarray(data).dtype == np.float64
    ip = np.ascontiguousarray(indptr, dtype=np.uint64)
    ix = np.ascontiguousarray(indices, dtype=np.uint64)
    d = np.ascontiguousarray(data)
    h = lib().or_op_csr(1 if f64 else 0, p(ip), p(ix), p(d), shape[0], shape[1])
    return Op(h, shape[0], f64)


def op_csr_i32(indptr, indices, data, shape, f64=True):
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    d = np.ascontiguousarray(data, dtype=np.float64)
    h = lib().or_op_csr_i32(1, p(ip), p(ix), p(d), shape[0], shape[1])
    op = Op(h, shape[0], True)
    if not f64:
        # an FP32 operator over the same arrays (values rounded to float)
        d32 = d.astype(np.float32)
        ip64 = ip.astype(np.uint64)
        ix64 = ix.astype(np.uint64)
        h32 = lib().or_op_csr(0, p(ip64), p(ix64), p(d32), shape[0], shape[1])
        return Op(h32, shape[0], False)
    return op


def op_identity(n, f64=True):
    return Op(lib().or_op_identity(1 if f64 else 0, n), n, f64)


def op_diagonal(d, f64=True):
    d = np.ascontiguousarray(d, dtype=np.float64 if f64 else np.float32)
    return Op(lib().or_op_diagonal(1 if f64 else 0, p(d), d.size), d.size, f64)


def op_jacobi(a: Op):
    e = Err()
    h = lib().or_op_jacobi(a.h, C.byref(e))
    if not h:
        raise ValueError(e.msg.decode())
    return Op(h, a.n, a.f64)


def op_ic0(a: Op, fast=True):
    e = Err()
    h = lib().or_op_ic0(a.h, 1 if fast else 0, C.byref(e))
    if not h:
        raise ValueError(e.msg.decode())
    return Op(h, a.n, a.f64)


def op_ilu0(a: Op):
    e = Err()
    h = lib().or_op_ilu0(a.h, C.byref(e))
    if not h:
        raise ValueError(e.msg.decode())
    return Op(h, a.n, a.f64)


def op_ssor(a: Op, omega: float):
    e = Err()
    h = lib().or_op_ssor(a.h, omega, C.byref(e))
    if not h:
        raise ValueError(e.msg.decode())
    op = Op(h, a.n, a.f64)
    op._base = a  # the SSOR operator reads a's arrays
    return op


def op_fsai(g: Op):
    return Op(lib().or_op_fsai(g.h), g.n, g.f64)


MESSAGES = [
    "Converged",
    "Maximum iterations reached",
    "Matrix not positive definite (p^T*A*p <= 0)",
    "Converged with initial guess",
    "BiCGSTAB breakdown: rho ≈ 0",
    "BiCGSTAB breakdown: (r_hat, v) ≈ 0",
    "BiCGSTAB breakdown: alpha is not finite",
    "BiCGSTAB breakdown: (t, t) ≈ 0",
    "BiCGSTAB breakdown: omega is not finite or too small",
    "BiCG breakdown: (p_star, q) ≈ 0",
    "BiCG breakdown: rho ≈ 0",
    "CGS breakdown: rho ≈ 0",
    "CGS breakdown: sigma ≈ 0",
    "Converged at initial guess",
    "Breakdown: rho = 0",
    "Breakdown: <p_tilde, q> = 0",
    "Converged in {iterations} iterations",
    "Breakdown: omega = 0",
    "Did not converge in {max_iter} iterations. Residual: {r}",
    "System has zero right-hand side",
    "Initial residual is zero",
]


def rust_display(v) -> str:
    """Rust's `{}` for an f64 / f32: shortest round-trip digits, no exponent."""
    if np.isnan(v):
        return "NaN"
    if np.isinf(v):
        return "-inf" if v < 0 else "inf"
    return np.format_float_positional(v, unique=True, trim="-")


def format_message(code, iterations, residual, f64=True):
    m = MESSAGES[code]
    r = rust_display(np.float64(residual) if f64 else np.float32(residual))
    return m.replace("{iterations}", str(iterations)).replace("{max_iter}", str(iterations)).replace("{r}", r)


def _solve(kind, a: Op, b, max_iter, rtol, atol, x0, m=None, m2=None, restart=30):
    dt = np.float64 if a.f64 else np.float32
    b = np.ascontiguousarray(b, dtype=dt)
    x = np.empty(a.n, dtype=dt)
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=dt)
    r, e = Res(), Err()
    L = lib()
    mh = m.h if m is not None else None
    if kind == "cg":
        rc = L.or_cg(a.h, p(b), max_iter, rtol, atol, p(x0a), mh, p(x), C.byref(r), C.byref(e))
    elif kind == "bicgstab":
        m2h = m2.h if m2 is not None else None
        rc = L.or_bicgstab(a.h, p(b), max_iter, rtol, atol, p(x0a), mh, m2h, p(x), C.byref(r), C.byref(e))
    elif kind == "gmres":
        rc = L.or_gmres(a.h, p(b), max_iter, restart, rtol, atol, p(x0a), mh, p(x), C.byref(r), C.byref(e))
    elif kind in ("bicg", "qmr"):
        m2h = m2.h if m2 is not None else None
        f = L.or_bicg if kind == "bicg" else L.or_qmr
        rc = f(a.h, p(b), max_iter, rtol, atol, p(x0a), mh, m2h, p(x), C.byref(r), C.byref(e))
    elif kind == "cgs":
        rc = L.or_cgs(a.h, p(b), max_iter, rtol, atol, p(x0a), mh, p(x), C.byref(r), C.byref(e))
    elif kind == "minres":
        rc = L.or_minres(a.h, p(b), max_iter, rtol, atol, p(x0a), mh, p(x), C.byref(r), C.byref(e))
    else:
        rc = L.or_lgmres(a.h, p(b), max_iter, restart, rtol, atol, p(x0a), mh, p(x), C.byref(r), C.byref(e))
    if rc:
        raise ValueError(e.msg.decode())
    return dict(x=x, iterations=int(r.iterations), residual_norm=float(r.residual_norm),
                converged=bool(r.converged),
                message=format_message(r.message, int(r.iterations), r.residual_norm, a.f64))


def cg(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, preconditioner=None):
    return _solve("cg", a, b, max_iter, rtol, atol, x0, preconditioner)


def bicgstab(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, left=None, right=None):
    return _solve("bicgstab", a, b, max_iter, rtol, atol, x0, left, right)


def gmres(a, b, max_iter=1000, restart=30, rtol=1e-8, atol=1e-12, x0=None, preconditioner=None):
    return _solve("gmres", a, b, max_iter, rtol, atol, x0, preconditioner, restart=restart)


def bicg(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, left=None, right=None):
    return _solve("bicg", a, b, max_iter, rtol, atol, x0, left, right)


def cgs(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, right=None):
    return _solve("cgs", a, b, max_iter, rtol, atol, x0, right)


def qmr(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, left=None, right=None):
    return _solve("qmr", a, b, max_iter, rtol, atol, x0, left, right)


def minres(a, b, max_iter=1000, rtol=1e-8, atol=1e-12, x0=None, preconditioner=None):
    return _solve("minres", a, b, max_iter, rtol, atol, x0, preconditioner)


def lgmres(a, b, max_iter=500, rtol=1e-8, atol=1e-8, inner_m=30, x0=None, preconditioner=None):
    return _solve("lgmres", a, b, max_iter, rtol, atol, x0, preconditioner, restart=inner_m)


def spmv_i32(indptr, indices, data, x):
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    f64 = np.asarray(data).dtype == np.float64
    data = np.ascontiguousarray(data)
    x = np.ascontiguousarray(x, dtype=data.dtype)
    y = np.empty(len(indptr) - 1, dtype=data.dtype)
    if f64:
        lib().or_spmv_i32_f64(p(indptr), p(indices), p(data), len(indptr) - 1, p(x), p(y))
    else:
        lib().or_spmv_i32_f32(p(indptr), p(indices), p(data), len(indptr) - 1, p(x), p(y))
    return y


def cg_mixed_ir(indptr, indices, data, b, tol=1e-10, inner_rtol=1e-4, max_outer=30,
                max_inner=10000, jacobi=True):
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = len(indptr) - 1
    x = np.empty(n, dtype=np.float64)
    o = IROpt(max_outer, max_inner, tol, inner_rtol, 1 if jacobi else 0)
    r = IRRes()
    lib().or_cg_mixed_ir(p(indptr), p(indices), p(data), n, p(b), C.byref(o), p(x), C.byref(r))
    return dict(x=x, outer=int(r.outer_iterations), inner=int(r.inner_iterations),
                rel_residual=float(r.rel_residual), converged=bool(r.converged))


def cg_mixed_replace(indptr, indices, data, b, tol=1e-10, delta=0.1, max_outer=30,
                     max_inner=10000, jacobi=True):
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = len(indptr) - 1
    x = np.empty(n, dtype=np.float64)
    o = IROpt(max_outer, max_inner, tol, 0.0, 1 if jacobi else 0)
    r = IRRes()
    lib().or_cg_mixed_replace(p(indptr), p(indices), p(data), n, p(b), C.byref(o), delta, p(x),
                              C.byref(r))
    return dict(x=x, outer=int(r.outer_iterations), inner=int(r.inner_iterations),
                rel_residual=float(r.rel_residual), converged=bool(r.converged))


def true_rel_residual(indptr, indices, data, b, x):
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().or_true_rel_residual(p(indptr), p(indices), p(data), len(indptr) - 1, p(b), p(x))


# ------------------------------------------------------ symmetric CSR (lower)
def _sym_arrays(indptr, indices, data):
    return (np.ascontiguousarray(indptr, dtype=np.uint64), np.ascontiguousarray(indices, dtype=np.uint64),
            np.ascontiguousarray(data))


def sym_check(data_len, indptr, indices, shape):
    """SymCsrMatrix::new validation: (code, message), code 0 = Ok."""
    indptr = np.ascontiguousarray(indptr, dtype=np.uint64)
    indices = np.ascontiguousarray(indices, dtype=np.uint64)
    e = Err()
    rc = lib().or_sym_csr_check(data_len, p(indptr), len(indptr), p(indices), len(indices),
                                int(shape[0]), int(shape[1]), C.byref(e))
    return rc, e.msg.decode()


def sym_matvec(indptr, indices, data, x):
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    n = len(indptr) - 1
    x = np.ascontiguousarray(x, dtype=data.dtype)
    y = np.empty(n, dtype=data.dtype)
    f = lib().or_sym_csr_matvec_f64 if data.dtype == np.float64 else lib().or_sym_csr_matvec_f32
    f(p(indptr), p(indices), p(data), n, p(x), p(y))
    return y


def sym_nnz(indptr, indices):
    indptr = np.ascontiguousarray(indptr, dtype=np.uint64)
    indices = np.ascontiguousarray(indices, dtype=np.uint64)
    return lib().or_sym_csr_nnz(p(indptr), p(indices), len(indices), len(indptr) - 1)


def sym_get(indptr, indices, data, i, j):
    indptr, indices, data = _sym_arrays(indptr, indices, np.asarray(data, dtype=np.float64))
    return lib().or_sym_csr_get_f64(p(indptr), p(indices), p(data), len(indptr) - 1, i, j)


def sym_trace(indptr, indices, data):
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    f = lib().or_sym_csr_trace_f64 if data.dtype == np.float64 else lib().or_sym_csr_trace_f32
    return data.dtype.type(f(p(indptr), p(indices), p(data), len(indptr) - 1))


def sym_quadratic_form(indptr, indices, data, x):
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    x = np.ascontiguousarray(x, dtype=data.dtype)
    f = (lib().or_sym_csr_quadratic_form_f64 if data.dtype == np.float64
         else lib().or_sym_csr_quadratic_form_f32)
    return data.dtype.type(f(p(indptr), p(indices), p(data), len(indptr) - 1, p(x)))


def sym_rank1_update(indptr, indices, data, x, alpha):
    """New (indptr, indices, data) of sym_csr_rank1_update."""
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    n = len(indptr) - 1
    x = np.ascontiguousarray(x, dtype=data.dtype)
    f = (lib().or_sym_csr_rank1_update_f64 if data.dtype == np.float64
         else lib().or_sym_csr_rank1_update_f32)
    cap = max(n * (n + 1) // 2, 1)
    ip = np.empty(n + 1, dtype=np.uint64)
    ix = np.empty(cap, dtype=np.uint64)
    dv = np.empty(cap, dtype=data.dtype)
    nnz = f(p(indptr), p(indices), p(data), n, p(x), alpha, p(ip), p(ix), p(dv))
    return ip, ix[:nnz].copy(), dv[:nnz].copy()


def sym_from_csr(indptr, indices, data, shape):
    """SymCsrMatrix::from_csr on CSR arrays: ((indptr, indices, data), None) or (None, message)."""
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    nr = int(shape[0])
    ip = np.empty(nr + 1, dtype=np.uint64)
    ix = np.empty(max(len(indices), 1), dtype=np.uint64)
    dv = np.empty(max(len(indices), 1), dtype=data.dtype)
    e = Err()
    f = lib().or_sym_csr_from_csr_f64 if data.dtype == np.float64 else lib().or_sym_csr_from_csr_f32
    rc = f(p(indptr), p(indices), p(data), nr, int(shape[1]), p(ip), p(ix), p(dv), C.byref(e))
    if rc:
        return None, e.msg.decode()
    nnz = int(ip[-1])
    return (ip, ix[:nnz].copy(), dv[:nnz].copy()), None


# ---------------------------------------------------------------- eigen
class OracleError(Exception):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def power_iteration(indptr, indices, data, max_iter=100, tol=1e-8, normalize=True, initial_guess=None):
    """power_iteration (eigen.rs:124-293) on SymCsrMatrix arrays."""
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    n = len(indptr) - 1
    f64 = data.dtype == np.float64
    x0 = None if initial_guess is None else np.ascontiguousarray(initial_guess, dtype=data.dtype)
    lam = np.zeros(1, dtype=data.dtype)
    res = np.zeros(1, dtype=data.dtype)
    vec = np.zeros(max(n, 1), dtype=data.dtype)
    info, e = EigInfo(), Err()
    f = lib().or_power_iteration_f64 if f64 else lib().or_power_iteration_f32
    rc = f(p(indptr), p(indices), p(data), n, max_iter, tol, 1 if normalize else 0, p(x0),
           0 if x0 is None else x0.size, p(lam), p(vec), p(res), C.byref(info), C.byref(e))
    if rc:
        raise OracleError(rc, e.msg.decode())
    return {"eigenvalues": lam, "eigenvectors": vec[:n].reshape(n, 1), "iterations": info.iterations,
            "residuals": res, "converged": bool(info.converged)}


def lanczos(indptr, indices, data, max_iter=1000, max_subspace_size=20, tol=1e-8, num_eigenvalues=1,
            compute_eigenvectors=True, initial_guess=None):
    """lanczos (eigen.rs:295-494) on SymCsrMatrix arrays."""
    indptr, indices, data = _sym_arrays(indptr, indices, data)
    n = len(indptr) - 1
    f64 = data.dtype == np.float64
    x0 = None if initial_guess is None else np.ascontiguousarray(initial_guess, dtype=data.dtype)
    k = max(min(num_eigenvalues, max_subspace_size, n), 1)
    vals = np.zeros(max(k, 3), dtype=data.dtype)
    res = np.zeros(k, dtype=data.dtype)
    vecs = np.zeros(max(n * k, 1), dtype=data.dtype)
    info, e = EigInfo(), Err()
    f = lib().or_lanczos_f64 if f64 else lib().or_lanczos_f32
    rc = f(p(indptr), p(indices), p(data), n, max_iter, max_subspace_size, tol, num_eigenvalues,
           1 if compute_eigenvectors else 0, p(x0), 0 if x0 is None else x0.size, p(vals), p(vecs), p(res),
           C.byref(info), C.byref(e))
    if rc:
        raise OracleError(rc, e.msg.decode())
    cols = int(info.num)
    return {"eigenvalues": vals[: int(info.count)].copy(),
            "eigenvectors": vecs[: n * cols].reshape(n, cols) if compute_eigenvectors else None,
            "iterations": info.iterations, "residuals": res[:cols].copy(), "converged": bool(info.converged)}


def tridiag_eig(alpha, beta, num):
    """solve_tridiagonal_eigenproblem (eigen.rs:512-646): (values, vectors) with
    vectors[k] the k-th eigenvector, or OracleError."""
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    m = len(alpha)
    vals = np.zeros(max(m, 3))
    vecs = np.zeros(max(m * max(m, 3), 1))
    cnt = C.c_uint64()
    e = Err()
    rc = lib().or_tridiag_eig_f64(p(alpha), p(beta) if len(beta) else None, m, len(beta), num, p(vals), p(vecs),
                                  C.byref(cnt), C.byref(e))
    if rc:
        raise OracleError(rc, e.msg.decode())
    c = int(cnt.value)
    return vals[:c].copy(), [vecs[k * m:(k + 1) * m].copy() for k in range(c)]


def solve_cubic(p_, q, r):
    """solve_cubic (eigen.rs:890-952): the roots it returns (1 or 3)."""
    roots = np.zeros(3)
    k = lib().or_solve_cubic_f64(p_, q, r, p(roots))
    return roots[:k].copy()


# ------------------------------------------------------------- host threads
def set_threads(n: int) -> None:
    """Host threads of the row-parallel SpMV and elementwise loops (results
    are bit-identical for any count; reductions stay serial)."""
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return int(lib().or_get_threads())


# ----------------------------------------------------- workload generators
GEN_KINDS = {"poisson2d": 0, "laplace3d": 1, "varcoef3d": 2, "varcoef2d": 3, "aniso_q1": 4, "powerlaw": 5}


def generate(kind: str, nx: int, ny: int = 1, nz: int = 1, seed: int = 0, param0: float = 0.0,
             param1: float = 0.0):
    """The library's seeded generators, restated on the CPU: (indptr int64,
    indices int32, values float64), bit-identical to scirs_gb300.generate."""
    n, nnz = C.c_int64(), C.c_int64()
    k = GEN_KINDS[kind]
    rc = lib().or_gen_matrix(k, nx, ny, nz, seed, param0, param1, C.byref(n), C.byref(nnz), None, None, None)
    if rc:
        raise ValueError(f"generator {kind} rejected its arguments ({rc})")
    indptr = np.empty(n.value + 1, dtype=np.int64)
    indices = np.empty(nnz.value, dtype=np.int32)
    vals = np.empty(nnz.value, dtype=np.float64)
    rc = lib().or_gen_matrix(k, nx, ny, nz, seed, param0, param1, C.byref(n), C.byref(nnz), p(indptr),
                             p(indices), p(vals))
    if rc:
        raise ValueError(f"generator {kind} failed ({rc})")
    return indptr, indices, vals


def rhs_normal(seed: int, n: int) -> np.ndarray:
    b = np.empty(n, dtype=np.float64)
    lib().or_gen_rhs_normal(seed, n, p(b))
    return b


def batch_sides(nsys: int, side_min: int, side_max: int, seed: int) -> np.ndarray:
    out = np.empty(nsys, dtype=np.int64)
    lib().or_gen_batch_sides(nsys, side_min, side_max, seed, p(out))
    return out


def batch_system(s: int, side: int, seed: int, sigma: float = 1.0):
    """System s of the batched workload, numbered from 0 (its own CSR)."""
    return generate("varcoef2d", side, side, 1, seed=int(lib().or_gen_batch_system_seed(seed, s)), param0=sigma)


def sample_problem(seed: int, sides=(64, 512)):
    """(side, eps, theta) of the anisotropic training distribution for a seed:
    side uniform in `sides`, eps = 10^U(0, 3), theta ~ U[0, pi)."""
    rng = np.random.default_rng(seed)
    side = int(rng.integers(sides[0], sides[1] + 1))
    eps = float(10.0 ** rng.uniform(0.0, 3.0))
    theta = float(rng.uniform(0.0, np.pi))
    return side, eps, theta
