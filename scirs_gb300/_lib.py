"""ctypes binding of the C ABI declared in include/scirs_sparse.h.

The shared library is built in-tree by scirs_gb300/build.py.  Importing this
module never builds or falls back to anything: if the library is missing the
import raises, so no code path can silently run without the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libscirs_sparse_gpu.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA library first "
        "(python -c 'import __graft_entry__ as g; g.build()')"
    )

lib = C.CDLL(LIB_PATH)

c_u64 = C.c_uint64
c_i64 = C.c_int64
c_vp = C.c_void_p
c_int = C.c_int
c_dbl = C.c_double
ctx_t = c_vp
op_t = c_vp

SX_F32, SX_F64 = 0, 1
SX_MEM_HOST, SX_MEM_DEVICE = 0, 1
SX_API_CSR_MATRIX, SX_API_CSR_ARRAY = 0, 1
SX_OP_CSR, SX_OP_IDENTITY, SX_OP_SCALED_IDENTITY, SX_OP_DIAGONAL = 0, 1, 2, 3
SX_OP_JACOBI, SX_OP_IC0, SX_OP_FSAI, SX_OP_HOST = 4, 5, 6, 7
SX_IC0_REFERENCE, SX_IC0_TEXTBOOK = 0, 1
SX_OP_ZERO, SX_OP_SUM, SX_OP_PRODUCT, SX_OP_SYM_CSR = 8, 9, 10, 11
SX_OP_ILU0, SX_OP_SSOR = 12, 13
SX_SPMV_EXACT = 1
SX_SPMV_SYM_HALF = 2


class ErrorInfo(C.Structure):
    _fields_ = [
        ("code", c_int),
        ("v0", c_u64),
        ("v1", c_u64),
        ("v2", c_u64),
        ("v3", c_u64),
        ("message", C.c_char * 512),
    ]


class IterResult(C.Structure):
    _fields_ = [
        ("iterations", c_u64),
        ("residual_norm", c_dbl),
        ("converged", c_int),
        ("message", c_int),
    ]


class CGOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("x0", c_vp),
        ("preconditioner", op_t),
    ]


class BiCGSTABOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("x0", c_vp),
        ("left_preconditioner", op_t),
        ("right_preconditioner", op_t),
    ]


class GMRESOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("restart", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("x0", c_vp),
        ("preconditioner", op_t),
    ]


class BiCGOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("x0", c_vp),
        ("left_preconditioner", op_t),
        ("right_preconditioner", op_t),
    ]


class MINRESOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("x0", c_vp),
        ("preconditioner", op_t),
    ]


class LGMRESOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("inner_m", c_u64),
        ("outer_k", c_u64),
        ("x0", c_vp),
        ("preconditioner", op_t),
    ]


class EigenResult(C.Structure):
    _fields_ = [
        ("iterations", c_u64),
        ("converged", C.c_int),
        ("num_eigenvalues", c_u64),
        ("num_columns", c_u64),
    ]


class PowerOptions(C.Structure):
    _fields_ = [("max_iter", c_u64), ("tol", c_dbl), ("normalize", C.c_int)]


class LanczosOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("max_subspace_size", c_u64),
        ("tol", c_dbl),
        ("num_eigenvalues", c_u64),
        ("compute_eigenvectors", C.c_int),
    ]


class IROptions(C.Structure):
    _fields_ = [
        ("max_outer", c_u64),
        ("max_inner", c_u64),
        ("tol", c_dbl),
        ("inner_rtol", c_dbl),
        ("x0", c_vp),
        ("preconditioner", op_t),
        ("a32", op_t),
        ("mode", c_int),
        ("reserved", c_int),
        ("replace_factor", c_dbl),
    ]


SX_IR_REPLACE = 0
SX_IR_RESTART = 1


class IRResult(C.Structure):
    _fields_ = [
        ("outer_iterations", c_u64),
        ("inner_iterations", c_u64),
        ("rel_residual", c_dbl),
        ("converged", c_int),
    ]


class GenSpec(C.Structure):
    _fields_ = [
        ("kind", c_int),
        ("nx", c_i64),
        ("ny", c_i64),
        ("nz", c_i64),
        ("seed", c_u64),
        ("param0", c_dbl),
        ("param1", c_dbl),
    ]


class BatchedOptions(C.Structure):
    _fields_ = [
        ("max_iter", c_u64),
        ("rtol", c_dbl),
        ("atol", c_dbl),
        ("inner_rtol", c_dbl),
        ("max_outer", c_u64),
    ]


class BatchedResult(C.Structure):
    _fields_ = [
        ("inner_iterations", c_u64),
        ("rel_residual", c_dbl),
        ("converged", c_int),
    ]


class BatchedSummary(C.Structure):
    _fields_ = [
        ("outer_iterations", c_u64),
        ("converged_systems", c_u64),
        ("max_inner_iterations", c_u64),
        ("total_inner_iterations", c_u64),
        ("worst_rel_residual", c_dbl),
        ("kernel_launches", c_u64),
        ("threads_per_block", C.c_uint32),
        ("blocks_per_sm", C.c_uint32),
    ]


HOST_MATVEC_FN = C.CFUNCTYPE(c_int, c_vp, c_vp, c_vp, c_u64)

P = C.POINTER
_SIGS = {
    "sx_last_error": (None, [P(ErrorInfo)]),
    "sx_status_string": (C.c_char_p, [c_int]),
    "sx_message_string": (C.c_char_p, [c_int]),
    "sx_ctx_create": (c_int, [c_int, P(ctx_t)]),
    "sx_ctx_create_on_stream": (c_int, [c_int, c_vp, P(ctx_t)]),
    "sx_ctx_destroy": (c_int, [ctx_t]),
    "sx_ctx_stream": (c_vp, [ctx_t]),
    "sx_ctx_synchronize": (c_int, [ctx_t]),
    "sx_ctx_kernel_launches": (c_u64, [ctx_t]),
    "sx_ctx_set_wait_limit": (c_int, [ctx_t, c_u64]),
    "sx_wait_selftest": (c_int, [ctx_t, P(c_u64)]),
    "sx_probe_gather_rate": (c_int, [ctx_t, c_int, c_u64, c_u64, P(C.c_double)]),
    "sx_ctx_set_cg_recurrence": (c_int, [ctx_t, c_int]),
    "sx_mem_cache_trim": (c_int, []),
    "sx_mem_cache_bytes": (c_u64, []),
    "sx_csr_from_triplets": (c_int, [ctx_t, c_int, c_int, c_vp, c_vp, c_vp, c_u64, c_u64, c_u64, c_int, P(op_t)]),
    "sx_csr_from_raw": (c_int, [ctx_t, c_int, c_int, c_vp, c_u64, c_vp, c_vp, c_u64, c_u64, c_u64, P(op_t)]),
    "sx_csr_from_raw_i32": (c_int, [ctx_t, c_int, c_vp, c_vp, c_vp, c_u64, c_u64, c_u64, c_int, P(op_t)]),
    "sx_csr_transpose": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_csr_save_npz": (c_int, [ctx_t, op_t, C.c_char_p]),
    "sx_csr_load_npz": (c_int, [ctx_t, c_int, C.c_char_p, P(op_t)]),
    "sx_csr_astype": (c_int, [ctx_t, op_t, c_int, P(op_t)]),
    "sx_csr_info": (c_int, [op_t, P(c_u64), P(c_u64), P(c_u64), P(c_int)]),
    "sx_csr_download": (c_int, [ctx_t, op_t, c_vp, c_vp, c_vp]),
    "sx_csr_get": (c_int, [ctx_t, op_t, c_u64, c_u64, c_vp]),
    "sx_op_identity": (c_int, [ctx_t, c_int, c_u64, P(op_t)]),
    "sx_op_scaled_identity": (c_int, [ctx_t, c_int, c_u64, c_dbl, P(op_t)]),
    "sx_op_diagonal": (c_int, [ctx_t, c_int, c_vp, c_u64, P(op_t)]),
    "sx_op_host": (c_int, [ctx_t, c_int, c_u64, c_u64, HOST_MATVEC_FN, c_vp, P(op_t)]),
    "sx_op_kind_of": (c_int, [op_t, P(c_int)]),
    "sx_op_shape": (c_int, [op_t, P(c_u64), P(c_u64)]),
    "sx_op_dtype": (c_int, [op_t, P(c_int)]),
    "sx_op_destroy": (c_int, [op_t]),
    "sx_op_matvec": (c_int, [ctx_t, op_t, c_vp, c_u64, c_vp, c_int]),
    "sx_op_rmatvec": (c_int, [ctx_t, op_t, c_vp, c_u64, c_vp, c_int]),
    "sx_spmv_ex": (c_int, [ctx_t, op_t, c_vp, c_vp, C.c_uint]),
    "sx_spmv_kernel": (c_int, [ctx_t, op_t, C.c_uint, C.c_char_p, c_u64]),
    "sx_op_zero": (c_int, [ctx_t, c_int, c_u64, c_u64, P(op_t)]),
    "sx_op_sum": (c_int, [ctx_t, op_t, op_t, P(op_t)]),
    "sx_op_product": (c_int, [ctx_t, op_t, op_t, P(op_t)]),
    "sx_op_has_adjoint": (c_int, [op_t, P(c_int)]),
    "sx_sym_csr_new": (c_int, [ctx_t, c_int, c_vp, c_u64, c_vp, c_u64, c_vp, c_u64, c_u64, c_u64, P(op_t)]),
    "sx_sym_csr_from_csr": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_sym_csr_info": (c_int, [ctx_t, op_t, P(c_u64), P(c_u64)]),
    "sx_sym_csr_download": (c_int, [ctx_t, op_t, c_vp, c_vp, c_vp]),
    "sx_sym_csr_to_csr": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_sym_csr_trace": (c_int, [ctx_t, op_t, c_vp]),
    "sx_sym_csr_quadratic_form": (c_int, [ctx_t, op_t, c_vp, c_u64, c_int, c_vp]),
    "sx_sym_csr_rank1_update": (c_int, [ctx_t, op_t, c_vp, c_u64, c_dbl, c_int]),
    "sx_precond_jacobi": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_precond_jacobi_from_diagonal": (c_int, [ctx_t, c_int, c_vp, c_u64, P(op_t)]),
    "sx_precond_ic0": (c_int, [ctx_t, op_t, c_int, P(op_t)]),
    "sx_precond_fsai": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_precond_ilu0": (c_int, [ctx_t, op_t, P(op_t)]),
    "sx_precond_ssor": (c_int, [ctx_t, op_t, c_dbl, P(op_t)]),
    "sx_cg_options_default": (None, [P(CGOptions)]),
    "sx_bicgstab_options_default": (None, [P(BiCGSTABOptions)]),
    "sx_gmres_options_default": (None, [P(GMRESOptions)]),
    "sx_cg": (c_int, [ctx_t, op_t, c_vp, c_u64, P(CGOptions), c_vp, c_int, P(IterResult)]),
    "sx_bicgstab": (c_int, [ctx_t, op_t, c_vp, c_u64, P(BiCGSTABOptions), c_vp, c_int, P(IterResult)]),
    "sx_gmres": (c_int, [ctx_t, op_t, c_vp, c_u64, P(GMRESOptions), c_vp, c_int, P(IterResult)]),
    "sx_bicg_options_default": (None, [P(BiCGOptions)]),
    "sx_minres_options_default": (None, [P(MINRESOptions)]),
    "sx_lgmres_options_default": (None, [P(LGMRESOptions)]),
    "sx_bicg": (c_int, [ctx_t, op_t, c_vp, c_u64, P(BiCGOptions), c_vp, c_int, P(IterResult)]),
    "sx_cgs": (c_int, [ctx_t, op_t, c_vp, c_u64, P(BiCGOptions), c_vp, c_int, P(IterResult)]),
    "sx_qmr": (c_int, [ctx_t, op_t, c_vp, c_u64, P(BiCGOptions), c_vp, c_int, P(IterResult)]),
    "sx_minres": (c_int, [ctx_t, op_t, c_vp, c_u64, P(MINRESOptions), c_vp, c_int, P(IterResult)]),
    "sx_lgmres": (c_int, [ctx_t, op_t, c_vp, c_u64, P(LGMRESOptions), c_vp, c_int, P(IterResult)]),
    "sx_power_options_default": (None, [P(PowerOptions)]),
    "sx_power_iteration": (c_int, [ctx_t, op_t, P(PowerOptions), c_vp, c_u64, c_int, c_vp, c_vp, c_vp,
                                   P(EigenResult)]),
    "sx_lanczos_options_default": (None, [P(LanczosOptions)]),
    "sx_tridiag_eig": (c_int, [c_vp, c_vp, c_u64, c_u64, c_u64, c_vp, c_vp, P(c_u64)]),
    "sx_lanczos": (c_int, [ctx_t, op_t, P(LanczosOptions), c_vp, c_u64, c_int, c_vp, c_vp, c_vp, P(EigenResult)]),
    "sx_iter_message": (c_int, [P(IterResult), c_int, C.c_char_p, c_u64]),
    "sx_ir_options_default": (None, [P(IROptions)]),
    "sx_cg_mixed": (c_int, [ctx_t, op_t, c_vp, c_u64, P(IROptions), c_vp, c_int, P(IRResult)]),
    "sx_true_rel_residual": (c_int, [ctx_t, op_t, c_vp, c_vp, c_int, P(c_dbl)]),
    "sx_true_rel_residual_noalloc": (c_int, [ctx_t, op_t, c_vp, c_vp, P(c_dbl)]),
    "sx_gen_matrix": (c_int, [P(GenSpec), P(c_i64), P(c_i64), c_vp, c_vp, c_vp]),
    "sx_gen_rhs_normal": (None, [c_u64, c_i64, c_vp]),
    "sx_gen_batch_varcoef2d": (c_int, [c_u64, c_i64, c_i64, c_u64, c_dbl, c_vp, P(c_i64), P(c_i64), c_vp, c_vp, c_vp]),
    "sx_batched_options_default": (None, [P(BatchedOptions)]),
    "sx_gnn_num_params": (c_u64, []),
    "sx_gnn_create": (c_int, [ctx_t, c_vp, c_u64, P(c_vp)]),
    "sx_gnn_destroy": (c_int, [c_vp]),
    "sx_gnn_get_params": (c_int, [ctx_t, c_vp, c_vp]),
    "sx_gnn_set_params": (c_int, [ctx_t, c_vp, c_vp]),
    "sx_gnn_loss_grad": (c_int, [ctx_t, c_vp, op_t, c_vp, c_u64, P(C.c_float), c_vp]),
    "sx_gnn_train_step": (c_int, [ctx_t, c_vp, op_t, c_u64, C.c_float, P(C.c_float)]),
    "sx_gnn_edge_values": (c_int, [ctx_t, c_vp, op_t, c_vp, P(c_u64)]),
    "sx_precond_learned": (c_int, [ctx_t, op_t, c_vp, P(op_t)]),
    "sx_batched_pcg": (c_int, [ctx_t, op_t, op_t, c_vp, c_u64, c_vp, c_vp, P(BatchedOptions), c_int,
                               c_vp, P(BatchedSummary)]),
}

MISSING = []
for _name, (_res, _args) in _SIGS.items():
    try:
        _f = getattr(lib, _name)
    except AttributeError:
        MISSING.append(_name)
        continue
    _f.restype = _res
    _f.argtypes = _args
