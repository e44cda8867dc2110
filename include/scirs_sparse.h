/* scirs_sparse.h -- C ABI of the GB300 sparse iterative-solve library.
 *
 * Drop-in device backend for the iterative-solve path of scirs2-sparse
 * (cool-japan/scirs, workspace 0.1.0-alpha.6): CSR construction and
 * transpose, CSR SpMV, the LinearOperator slot (operators and
 * preconditioners), and the cg / bicgstab / gmres solvers.  Every entry point
 * names the reference item it replaces (paths relative to the reference
 * workspace).  A Rust shim can implement the crate's traits on top of these
 * calls.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Indices cross the boundary as uint64_t
 *    (Rust usize); the device keeps int32 indices and rejects larger values
 *    with SX_ERR_INDEX_CAST_OVERFLOW (index_dtype.rs:109-170 semantics).
 *  - Values are float (SX_F32) or double (SX_F64); `const void*` value
 *    pointers point at the dtype of the handle they go with.
 *  - `mem` arguments say where vector buffers live: SX_MEM_HOST (pageable or
 *    pinned host memory, copied in/out inside the call) or SX_MEM_DEVICE
 *    (device pointers on the context's device, used in place).
 *  - Calls are synchronous on the context's stream, like the reference's
 *    blocking calls.  Handles are not thread-safe: one context per thread.
 *  - Errors: a non-zero sx_status; sx_last_error() returns the structured
 *    payload and the SparseError Display string for the calling thread.
 *  - Solver non-convergence and breakdown are NOT errors: they return SX_OK
 *    with converged = 0 and a message code, as IterationResult does.
 */
#ifndef SCIRS_SPARSE_H
#define SCIRS_SPARSE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
/* 1..14 follow SparseError's variants in declaration order
 * (scirs2-sparse/src/error.rs:9-74). */
typedef enum {
  SX_OK = 0,
  SX_ERR_COMPUTATION = 1,             /* ComputationError(String)            */
  SX_ERR_DIMENSION_MISMATCH = 2,      /* DimensionMismatch{expected, found}  */
  SX_ERR_INDEX_OUT_OF_BOUNDS = 3,     /* IndexOutOfBounds{index, shape}      */
  SX_ERR_INVALID_AXIS = 4,            /* InvalidAxis                          */
  SX_ERR_INVALID_SLICE_RANGE = 5,     /* InvalidSliceRange                    */
  SX_ERR_INCONSISTENT_DATA = 6,       /* InconsistentData{reason}            */
  SX_ERR_NOT_IMPLEMENTED = 7,         /* NotImplemented(String)              */
  SX_ERR_SINGULAR_MATRIX = 8,         /* SingularMatrix(String)              */
  SX_ERR_VALUE = 9,                   /* ValueError(String)                  */
  SX_ERR_CONVERSION = 10,             /* ConversionError(String)             */
  SX_ERR_OPERATION_NOT_SUPPORTED = 11,/* OperationNotSupported(String)       */
  SX_ERR_SHAPE_MISMATCH = 12,         /* ShapeMismatch{expected, found}      */
  SX_ERR_ITERATIVE_SOLVER_FAILURE = 13,/* IterativeSolverFailure(String)     */
  SX_ERR_INDEX_CAST_OVERFLOW = 14,    /* IndexCastOverflow{value, target}    */
  /* device-side conditions with no SparseError counterpart */
  SX_ERR_CUDA = 100,                  /* a CUDA runtime call failed           */
  SX_ERR_DEVICE_TIMEOUT = 101,        /* a bounded device-side wait ran out   */
  SX_ERR_INVALID_ARGUMENT = 102,      /* null handle, bad enum, dtype clash   */
  SX_ERR_OUT_OF_MEMORY = 103          /* device allocation failed             */
} sx_status;

typedef struct {
  int code;          /* sx_status */
  uint64_t v0, v1;   /* DimensionMismatch: expected, found; IndexOutOfBounds: index (r, c);
                        IndexCastOverflow: value */
  uint64_t v2, v3;   /* IndexOutOfBounds / ShapeMismatch: shape (r, c) */
  char message[512]; /* the SparseError Display text, e.g.
                        "Value error: Row index out of bounds" */
} sx_error_info;

/* Last error of the calling thread (copies into *out). */
void sx_last_error(sx_error_info* out);
const char* sx_status_string(int status);

typedef enum { SX_F32 = 0, SX_F64 = 1 } sx_dtype;
typedef enum { SX_MEM_HOST = 0, SX_MEM_DEVICE = 1 } sx_mem;

/* ----------------------------------------------------------------- context */
typedef struct sx_ctx_s* sx_ctx;

/* A context owns a non-blocking CUDA stream, reusable scratch space and the
 * SpMV autotune cache.  (No reference counterpart: the reference runs on the
 * caller's thread.) */
int sx_ctx_create(int device, sx_ctx* out);
/* Same, but work is enqueued on a caller-owned stream (cudaStream_t). */
int sx_ctx_create_on_stream(int device, void* stream, sx_ctx* out);
int sx_ctx_destroy(sx_ctx ctx);
void* sx_ctx_stream(sx_ctx ctx);
int sx_ctx_synchronize(sx_ctx ctx);

/* Time limit of one dependency wait inside the triangular factorisations
 * and sweeps (IC(0), ILU(0), SSOR) of this context, in nanoseconds; 0
 * restores the default of 2 s.  A wait that runs longer gives up, every
 * other wait of that launch ends at once, and the call reports
 * SX_ERR_DEVICE_TIMEOUT; the context and its other handles stay usable.  A
 * limit applies to launches made after it is set (solver graphs captured
 * earlier keep the limit they were captured with).  No reference
 * counterpart: the reference's triangular solves are sequential host loops. */
int sx_ctx_set_wait_limit(sx_ctx ctx, uint64_t ns);

/* One bounded device wait on a flag that nothing sets, with this context's
 * limit: returns SX_ERR_DEVICE_TIMEOUT when the wait gives up (the expected
 * outcome) and the wait's length in *waited_ns.  Checks the give-up path of
 * the dependency waits without touching any operator. */
int sx_wait_selftest(sx_ctx ctx, uint64_t* waited_ns);
/* CG variant of this context (on != 0): with a Jacobi, diagonal, scaled or no
 * preconditioner, sx_cg carries A p by the recurrence q = A z + beta q
 * (z = M r), so that each iteration takes two device kernels instead of
 * three (the p-update runs in the SpMV's epilogue, z = M r in the vector
 * update).  Mathematically the reference's loop (linalg/iterative.rs:95-151)
 * with the same roundings elsewhere; q differs from A p by the recurrence's
 * rounding, so iterates and iteration counts can differ slightly from the
 * reference's.  Off (0) by default; applies to solves started after it is
 * set.  No reference counterpart. */
int sx_ctx_set_cg_recurrence(sx_ctx ctx, int on);
/* Roofline probe: the rate (gathers per second) at which this GPU reads
 * elements of an L2-resident vector of n elements (dtype SX_F32 or SX_F64)
 * at m uniform random positions, the positions streamed with coalesced
 * loads.  SpMV on matrices with scattered columns (power-law graphs) is
 * bound by this rate rather than by HBM.  Allocates (n elements, m + a few
 * MB) and synchronises.  No reference counterpart. */
int sx_probe_gather_rate(sx_ctx ctx, sx_dtype dtype, uint64_t n, uint64_t m, double* gathers_per_s);
/* Number of kernels this library launched on the context (graph-launched
 * kernels included), for launch accounting. */
uint64_t sx_ctx_kernel_launches(sx_ctx ctx);

/* Device memory the library freed is held for reuse (up to 4 GiB per GPU;
 * a block is reused only after the work queued on every context stream of
 * its GPU at the time of the free has completed; SX_MEM_CACHE=0 in the
 * environment turns this off).  sx_mem_cache_trim returns every held block
 * to the CUDA driver; sx_mem_cache_bytes reports how much is held.  No
 * reference counterpart: the reference's arrays live in host memory. */
int sx_mem_cache_trim(void);
uint64_t sx_mem_cache_bytes(void);

/* --------------------------------------------------------------- operators */
/* One handle type for matrices, operators and preconditioners: the
 * reference's preconditioner slot is itself Box<dyn LinearOperator<F>>
 * (linalg/interface.rs:13-52, linalg/iterative.rs:17-23). */
typedef struct sx_op_s* sx_op;

typedef enum {
  SX_OP_CSR = 0,             /* MatrixLinearOperator<F, CsrMatrix<F>>  interface.rs:232-296 */
  SX_OP_IDENTITY = 1,        /* IdentityOperator                       interface.rs:55-93   */
  SX_OP_SCALED_IDENTITY = 2, /* ScaledIdentityOperator                 interface.rs:95-130  */
  SX_OP_DIAGONAL = 3,        /* DiagonalOperator                       interface.rs:132-175 */
  SX_OP_JACOBI = 4,          /* JacobiPreconditioner                   preconditioners.rs:14-92 */
  SX_OP_IC0 = 5,             /* IC0Preconditioner                      ic.rs:15-230 */
  SX_OP_FSAI = 6,            /* M^-1 = G G^T (learned factorised SAI; no reference counterpart) */
  SX_OP_HOST = 7,            /* user operator called back on the host  (dyn LinearOperator) */
  SX_OP_ZERO = 8,            /* ZeroOperator                           interface.rs:177-222 */
  SX_OP_SUM = 9,             /* SumOperator: (A + B) x                 interface.rs:299-349 */
  SX_OP_PRODUCT = 10,        /* ProductOperator: A (B x)               interface.rs:351-402 */
  SX_OP_SYM_CSR = 11,        /* SymCsrMatrix (lower triangle stored)   sym_csr.rs:24-337 */
  SX_OP_ILU0 = 12,           /* ILU0Preconditioner                     preconditioners.rs:194-399 */
  SX_OP_SSOR = 13            /* SSORPreconditioner                     preconditioners.rs:94-192 */
} sx_op_kind;

/* Which reference constructor's validation and error semantics to follow. */
typedef enum {
  SX_API_CSR_MATRIX = 0, /* CsrMatrix::new / from_raw_csr   csr.rs:92-227         */
  SX_API_CSR_ARRAY = 1   /* CsrArray::from_triplets / new   csr_array.rs:77-219   */
} sx_csr_api;

/* Triplets -> CSR on the device: validation, stable sort by (row, col) with
 * duplicates kept, row pointers by count + prefix sum.  Bit-exact with
 * CsrMatrix::new (csr.rs:92-160) or CsrArray::from_triplets(.., sorted)
 * (csr_array.rs:152-219).  rows/cols/data are host arrays of length nnz. */
int sx_csr_from_triplets(sx_ctx ctx, sx_dtype dtype, sx_csr_api api, const uint64_t* rows,
                         const uint64_t* cols, const void* data, uint64_t nnz, uint64_t nrows,
                         uint64_t ncols, int sorted, sx_op* out);

/* Raw CSR arrays (host): validation of CsrMatrix::from_raw_csr
 * (csr.rs:174-227) or CsrArray::new (csr_array.rs:77-136); arrays are kept
 * as given.  indptr has indptr_len entries, indices/data have nnz. */
int sx_csr_from_raw(sx_ctx ctx, sx_dtype dtype, sx_csr_api api, const uint64_t* indptr,
                    uint64_t indptr_len, const uint64_t* indices, const void* data, uint64_t nnz,
                    uint64_t nrows, uint64_t ncols, sx_op* out);

/* Device-native upload: int64 row pointers, int32 columns, values of
 * `dtype`, in host or device memory.  Validated like from_raw_csr.  (No
 * reference counterpart: saves the usize->int32 narrowing pass.) */
int sx_csr_from_raw_i32(sx_ctx ctx, sx_dtype dtype, const int64_t* indptr, const int32_t* indices,
                        const void* data, uint64_t nrows, uint64_t ncols, uint64_t nnz,
                        sx_mem mem, sx_op* out);

/* save_npz (io.rs:49-177) of a CSR operator: the reference's little-endian
 * "csr_array" record (format marker, shape, data, indices, indptr), not a
 * SciPy zip archive.  I/O failures: ComputationError "IO error: ...". */
int sx_csr_save_npz(sx_ctx ctx, sx_op a, const char* path);
/* load_npz (io.rs:197-269) of a "csr_array" record into a device CSR, with
 * CsrArray::new's validation (csr_array.rs:77-136); values are read in
 * `dtype`'s width, as load_npz::<T> does.  Other known markers (csc_array,
 * coo_array, dok_array) are NotImplemented; unknown ones ConversionError
 * "Unknown format: ..."; short files ComputationError "IO error: failed to
 * fill whole buffer". */
int sx_csr_load_npz(sx_ctx ctx, sx_dtype dtype, const char* path, sx_op* out);

/* Counting-sort transpose, bit-exact with CsrMatrix::transpose
 * (csr.rs:289-326) and CsrArray::transpose (csr_array.rs:595-625). */
int sx_csr_transpose(sx_ctx ctx, sx_op a, sx_op* out);

/* Value-type conversion of a CSR matrix (e.g. the FP32 copy used by the
 * mixed-precision solver).  No reference counterpart. */
int sx_csr_astype(sx_ctx ctx, sx_op a, sx_dtype dtype, sx_op* out);

/* CSR accessors: shape/nnz (csr.rs:244-264), arrays back to the host as
 * usize (the public indptr/indices/data fields, csr.rs:20-25), get(i, j)
 * with first-match semantics (csr.rs:33-48), has_sorted_indices
 * (csr_array.rs:221-233). */
int sx_csr_info(sx_op a, uint64_t* nrows, uint64_t* ncols, uint64_t* nnz, int* has_sorted_indices);
int sx_csr_download(sx_ctx ctx, sx_op a, uint64_t* indptr, uint64_t* indices, void* data);
int sx_csr_get(sx_ctx ctx, sx_op a, uint64_t i, uint64_t j, void* out_value);

int sx_op_identity(sx_ctx ctx, sx_dtype dtype, uint64_t n, sx_op* out);
int sx_op_scaled_identity(sx_ctx ctx, sx_dtype dtype, uint64_t n, double scale, sx_op* out);
int sx_op_diagonal(sx_ctx ctx, sx_dtype dtype, const void* diag, uint64_t n, sx_op* out);

/* Host-callback operator for a user-defined LinearOperator: the library
 * stages x to the host, calls fn(user, x, y, n), and copies y back.  The
 * solver loop itself stays on the device. */
typedef int (*sx_host_matvec_fn)(void* user, const void* x, void* y, uint64_t n);
int sx_op_host(sx_ctx ctx, sx_dtype dtype, uint64_t nrows, uint64_t ncols, sx_host_matvec_fn fn,
               void* user, sx_op* out);

int sx_op_kind_of(sx_op op, int* kind);
int sx_op_shape(sx_op op, uint64_t* nrows, uint64_t* ncols);
int sx_op_dtype(sx_op op, int* dtype);
int sx_op_destroy(sx_op op);

/* ZeroOperator::new(rows, cols) (interface.rs:184-191): matvec gives zeros. */
int sx_op_zero(sx_ctx ctx, sx_dtype dtype, uint64_t nrows, uint64_t ncols, sx_op* out);
/* SumOperator::new(a, b) (interface.rs:306-316; ShapeMismatch when the shapes
 * differ) and ProductOperator::new(a, b) (interface.rs:358-370;
 * DimensionMismatch when a's columns differ from b's rows).  The composite
 * borrows a and b (the reference takes ownership of boxes): they must
 * outlive it, and destroying it leaves them alone. */
int sx_op_sum(sx_ctx ctx, sx_op a, sx_op b, sx_op* out);
int sx_op_product(sx_ctx ctx, sx_op a, sx_op b, sx_op* out);
/* LinearOperator::has_adjoint (interface.rs:49-51 and each operator). */
int sx_op_has_adjoint(sx_op op, int* out);
/* y = A x (LinearOperator::matvec, interface.rs:18; CSR: interface.rs:257-279,
 * CsrArray::dot_vector csr_array.rs:569-593, CsrMatrix::dot csr.rs:479-497).
 * x has x_len entries (DimensionMismatch otherwise), y has nrows. */
int sx_op_matvec(sx_ctx ctx, sx_op op, const void* x, uint64_t x_len, void* y, sx_mem mem);
/* y = A^T x (LinearOperator::rmatvec; CSR: interface.rs:281-285, through a
 * cached device transpose instead of a transpose per call). */
int sx_op_rmatvec(sx_ctx ctx, sx_op op, const void* x, uint64_t x_len, void* y, sx_mem mem);

/* SpMV flags for sx_spmv_ex */
#define SX_SPMV_EXACT 1u /* per-row sequential sum of rounded products (reference order) */
#define SX_SPMV_SYM_HALF 2u /* symmetric operators: read only the stored lower triangle and
                             * add the transposed terms atomically (order not fixed) */
/* Device-pointer SpMV with an explicit summation mode, asynchronous on the
 * context stream.  flags = SX_SPMV_EXACT: the reference's rounding, bit for
 * bit (the mode of sx_op_matvec); flags = 0: FP64 rows are summed with fused
 * multiply-adds in storage order (a few ulp per row, half the FP64 pipe
 * work); FP32 is always exact.  SX_SPMV_SYM_HALF (symmetric operators
 * only, without SX_SPMV_EXACT) reads each stored entry once and scatters the
 * transposed terms with atomic adds: fewer bytes, but the summation order
 * varies from run to run (within a few ulp of the exact result). */
int sx_spmv_ex(sx_ctx ctx, sx_op a, const void* x_dev, void* y_dev, unsigned flags);
/* Name of the kernel sx_spmv_ex(flags) launches for `a` (diagnostics; no
 * reference counterpart), NUL-terminated into buf[len]. */
int sx_spmv_kernel(sx_ctx ctx, sx_op a, unsigned flags, char* buf, uint64_t len);

/* ------------------------------------------- symmetric CSR (lower storage) */
/* SymCsrMatrix::new(data, indptr, indices, (nrows, ncols)) (sym_csr.rs:64-134):
 * ValueError "Symmetric matrix must be square", "indptr length (a) must be
 * equal to rows + 1 (b)", "data length (a) must match indices length (b)",
 * "Last indptr value (a) must equal nnz (b)", IndexOutOfBounds for a column
 * >= ncols, ValueError "Symmetric CSR should only store the lower triangular
 * part"; in that order.  (A decreasing or overrunning indptr, a panic in the
 * reference, is InconsistentData.)  nnz = indices length.  The operator
 * applies the full symmetric matrix: sx_op_matvec / sx_spmv_ex give
 * sym_csr_matvec's result (sym_ops.rs:56-90) bit for bit; it works as A in
 * every solver and as its own adjoint; sx_csr_get gives SymCsrMatrix::get
 * (sym_csr.rs:280-298). */
int sx_sym_csr_new(sx_ctx ctx, sx_dtype dtype, const void* data, uint64_t data_len,
                   const uint64_t* indptr, uint64_t indptr_len, const uint64_t* indices,
                   uint64_t nnz, uint64_t nrows, uint64_t ncols, sx_op* out);
/* SymCsrMatrix::from_csr (sym_csr.rs:149-189): ValueError "Matrix must be
 * symmetric to convert to SymCSR format" when some stored |a_ij - get(j, i)|
 * exceeds 100 epsilon; else the col <= row entries in storage order. */
int sx_sym_csr_from_csr(sx_ctx ctx, sx_op a, sx_op* out);
/* nnz_stored (sym_csr.rs:241-243) and nnz (sym_csr.rs:254-268: rows that
 * store a diagonal entry count once, every other stored entry twice). */
int sx_sym_csr_info(sx_ctx ctx, sx_op a, uint64_t* nnz_stored, uint64_t* nnz_full);
/* The stored arrays (the public data/indptr/indices fields), as usize. */
int sx_sym_csr_download(sx_ctx ctx, sx_op a, uint64_t* indptr, uint64_t* indices, void* data);
/* SymCsrMatrix::to_csr (sym_csr.rs:305-337): a CsrMatrix of the full matrix. */
int sx_sym_csr_to_csr(sx_ctx ctx, sx_op a, sx_op* out);
/* sym_csr_trace (sym_ops.rs:317-335) and sym_csr_quadratic_form
 * (sym_ops.rs:271-283), summed in the reference's sequential order: bit for
 * bit.  x has x_len entries (DimensionMismatch otherwise). */
int sx_sym_csr_trace(sx_ctx ctx, sx_op a, void* out_value);
int sx_sym_csr_quadratic_form(sx_ctx ctx, sx_op a, const void* x, uint64_t x_len, sx_mem mem,
                              void* out_value);
/* sym_csr_rank1_update (sym_ops.rs:179-233): A = A + alpha x x^T in place
 * (lower triangle of the dense sum, zeros dropped; O(n^2) work as in the
 * reference).  alpha is converted to the operator's value type. */
int sx_sym_csr_rank1_update(sx_ctx ctx, sx_op a, const void* x, uint64_t x_len, double alpha,
                            sx_mem mem);

/* --------------------------------------------------------- preconditioners */
/* JacobiPreconditioner::new (preconditioners.rs:21-44): 1/get(i,i) with the
 * FIRST duplicate's value; ValueError "Zero diagonal element at position i"
 * when |d| < epsilon. */
int sx_precond_jacobi(sx_ctx ctx, sx_op a, sx_op* out);
/* JacobiPreconditioner::from_diagonal (preconditioners.rs:47-62). */
int sx_precond_jacobi_from_diagonal(sx_ctx ctx, sx_dtype dtype, const void* diag, uint64_t n,
                                    sx_op* out);

typedef enum {
  SX_IC0_REFERENCE = 0, /* the reference factorisation, ic.rs:22-135, bit-exact */
  SX_IC0_TEXTBOOK = 1   /* standard IC(0): L_ij = (a_ij - sum) / L_jj, d_i = sqrt(a_ii - sum L_ik^2) */
} sx_ic0_variant;
/* IC0Preconditioner::new (ic.rs:22-135) and its apply (ic.rs:143-220). */
int sx_precond_ic0(sx_ctx ctx, sx_op a, int variant, sx_op* out);

/* ILU0Preconditioner::new (preconditioners.rs:209-324) and its apply
 * (:331-375): the reference's factorisation order and rounding, bit for bit
 * (rows factorised in dependency order on the device); ValueError "Missing
 * diagonal element at row k" / "Zero pivot at position k" for the first
 * failing row.  The apply solves L y = x (unit diagonal), then U z = y
 * dividing by the last diagonal entry of each row.  Not self-adjoint:
 * rmatvec is OperationNotSupported.  A must be square (DimensionMismatch). */
int sx_precond_ilu0(sx_ctx ctx, sx_op a, sx_op* out);
/* SSORPreconditioner::new(matrix, omega) (preconditioners.rs:103-131) and
 * its apply (:140-187): forward sweep (D + omega L) y = x, z = y * D (as the
 * reference writes it), backward sweep (D + omega U) w = z; ValueError
 * "Relaxation parameter omega must be in (0, 2)" / "Zero diagonal element
 * at position i" (first diagonal entry, |d| < epsilon).  Not self-adjoint. */
int sx_precond_ssor(sx_ctx ctx, sx_op a, double omega, sx_op* out);

/* Factorised approximate inverse M^-1 = G G^T from a lower-triangular CSR G
 * (no reference counterpart; apply = two SpMVs through a cached G^T). */
int sx_precond_fsai(sx_ctx ctx, sx_op g, sx_op* out);

/* ----------------------------------------------------------------- solvers */
typedef enum {
  SX_MSG_CONVERGED = 0,           /* "Converged" */
  SX_MSG_MAX_ITER = 1,            /* "Maximum iterations reached" */
  SX_MSG_NOT_POSITIVE_DEFINITE = 2,/* "Matrix not positive definite (p^T*A*p <= 0)" */
  SX_MSG_CONVERGED_INITIAL = 3,   /* "Converged with initial guess" */
  SX_MSG_BREAKDOWN_RHO = 4,       /* "BiCGSTAB breakdown: rho ≈ 0" */
  SX_MSG_BREAKDOWN_RHAT_V = 5,    /* "BiCGSTAB breakdown: (r_hat, v) ≈ 0" */
  SX_MSG_BREAKDOWN_ALPHA = 6,     /* "BiCGSTAB breakdown: alpha is not finite" */
  SX_MSG_BREAKDOWN_TT = 7,        /* "BiCGSTAB breakdown: (t, t) ≈ 0" */
  SX_MSG_BREAKDOWN_OMEGA = 8,     /* "BiCGSTAB breakdown: omega is not finite or too small" */
  SX_MSG_BICG_PQ = 9,             /* "BiCG breakdown: (p_star, q) ≈ 0"       iterative.rs:276 */
  SX_MSG_BICG_RHO = 10,           /* "BiCG breakdown: rho ≈ 0"               iterative.rs:321 */
  SX_MSG_CGS_RHO = 11,            /* "CGS breakdown: rho ≈ 0"                cgs.rs:94 */
  SX_MSG_CGS_SIGMA = 12,          /* "CGS breakdown: sigma ≈ 0"              cgs.rs:131 */
  SX_MSG_QMR_INITIAL = 13,        /* "Converged at initial guess"            qmr.rs:105 */
  SX_MSG_QMR_RHO = 14,            /* "Breakdown: rho = 0"                    qmr.rs:124 */
  SX_MSG_QMR_PQ = 15,             /* "Breakdown: <p_tilde, q> = 0"           qmr.rs:184 */
  SX_MSG_QMR_CONVERGED = 16,      /* "Converged in {iterations} iterations"  qmr.rs:233 */
  SX_MSG_QMR_OMEGA = 17,          /* "Breakdown: omega = 0"                  qmr.rs:244 */
  SX_MSG_QMR_MAX_ITER = 18,       /* "Did not converge in {max_iter} iterations. Residual: {r}" qmr.rs:255 */
  SX_MSG_ZERO_RHS = 19,           /* "System has zero right-hand side"       minres.rs:99 */
  SX_MSG_ZERO_RESIDUAL = 20       /* "Initial residual is zero"              minres.rs:128 */
} sx_message;
/* The exact message strings of the reference (UTF-8); the two messages with
 * fields read "{iterations}" / "{max_iter}" / "{r}" here (sx_iter_message
 * fills them). */
const char* sx_message_string(int message);

/* IterationResult (iterative.rs:8-14); x is returned through x_out. */
typedef struct {
  uint64_t iterations;
  double residual_norm;
  int converged;
  int message; /* sx_message */
} sx_iter_result;

/* The result's message as the reference formats it, with the iteration
 * count and the residual (Rust `{}` formatting of an f64 / f32 by dtype) put
 * into the two QMR messages; NUL-terminated into buf[len]. */
int sx_iter_message(const sx_iter_result* res, int dtype, char* buf, uint64_t len);

/* CGOptions (iterative.rs:17-35); defaults: 1000, 1e-8, 1e-12, none, none. */
typedef struct {
  uint64_t max_iter;
  double rtol;
  double atol;
  const void* x0;      /* NULL = zeros; lives in `mem` like b */
  sx_op preconditioner;/* NULL = none */
} sx_cg_options;
/* BiCGSTABOptions (iterative.rs:348-368). */
typedef struct {
  uint64_t max_iter;
  double rtol;
  double atol;
  const void* x0;
  sx_op left_preconditioner;
  sx_op right_preconditioner;
} sx_bicgstab_options;
/* GMRESOptions (iterative.rs:614-634); restart default 30. */
typedef struct {
  uint64_t max_iter;
  uint64_t restart;
  double rtol;
  double atol;
  const void* x0;
  sx_op preconditioner;
} sx_gmres_options;

void sx_cg_options_default(sx_cg_options* o);
void sx_bicgstab_options_default(sx_bicgstab_options* o);
void sx_gmres_options_default(sx_gmres_options* o);

/* cg (iterative.rs:40-162).  b has b_len entries; x_out has nrows(a). */
int sx_cg(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_cg_options* opt,
          void* x_out, sx_mem mem, sx_iter_result* res);
/* bicgstab (iterative.rs:377-611). */
int sx_bicgstab(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len,
                const sx_bicgstab_options* opt, void* x_out, sx_mem mem, sx_iter_result* res);
/* gmres (iterative.rs:641-816).  Where the reference's loop would repeat a
 * cycle forever without progress, the call returns instead: restart = 0 with
 * SX_ERR_VALUE, a breakdown at a cycle's first Arnoldi step (A r0 parallel
 * to r0, e.g. A = 2 I) with SX_ERR_COMPUTATION; x_out is then not written. */
int sx_gmres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_gmres_options* opt,
             void* x_out, sx_mem mem, sx_iter_result* res);

/* BiCGOptions (iterative.rs:164-185), also CGSOptions (cgs.rs:8) and the
 * fields of QMROptions (qmr.rs:18-38); defaults: 1000, 1e-8, 1e-12, none,
 * none, none. */
typedef struct {
  uint64_t max_iter;
  double rtol;
  double atol;
  const void* x0;
  sx_op left_preconditioner;
  sx_op right_preconditioner;
} sx_bicg_options;
void sx_bicg_options_default(sx_bicg_options* o);
/* bicg (iterative.rs:189-345): needs A's adjoint (rmatvec). */
int sx_bicg(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt,
            void* x_out, sx_mem mem, sx_iter_result* res);
/* cgs (cgs.rs:15-193): only the right preconditioner is used. */
int sx_cgs(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt,
           void* x_out, sx_mem mem, sx_iter_result* res);
/* qmr (qmr.rs:44-259): needs A's adjoint (and the preconditioners').
 * DimensionMismatch{expected: b_len, found: rows} unless A is b_len x b_len. */
int sx_qmr(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt,
           void* x_out, sx_mem mem, sx_iter_result* res);

/* MINRESOptions (minres.rs:17-35); defaults: 1000, 1e-8, 1e-12, none, none. */
typedef struct {
  uint64_t max_iter;
  double rtol;
  double atol;
  const void* x0;
  sx_op preconditioner;
} sx_minres_options;
void sx_minres_options_default(sx_minres_options* o);
/* minres (minres.rs:66-257).  ComputationError "Indefinite preconditioner" /
 * "Non-symmetric matrix" when r' M r < 0. */
int sx_minres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_minres_options* opt,
              void* x_out, sx_mem mem, sx_iter_result* res);

/* LGMRESOptions (lgmres.rs:10-38); defaults: 500, 1e-8, 1e-8, 30, 3, none,
 * none.  outer_k is accepted and, as in the reference, does not change the
 * iteration (its augmentation vectors are never used). */
typedef struct {
  uint64_t max_iter;
  double rtol;
  double atol;
  uint64_t inner_m;
  uint64_t outer_k;
  const void* x0;
  sx_op preconditioner;
} sx_lgmres_options;
void sx_lgmres_options_default(sx_lgmres_options* o);
/* lgmres (lgmres.rs:58-188, inner cycle 191-327): iterations = outer cycles; inner_m <= 64.
 * LGMRESResult has no message: converged -> SX_MSG_CONVERGED, else
 * SX_MSG_MAX_ITER. */
int sx_lgmres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_lgmres_options* opt,
              void* x_out, sx_mem mem, sx_iter_result* res);

/* ------------------------------------------------ eigenpairs (eigen.rs)
 * Both take a symmetric CSR operator (sx_sym_csr_*), as the reference takes
 * a SymCsrMatrix.  x0 / v0 (NULL: e_0, as the reference) and the
 * eigenvector output are host or device memory per `mem`; eigenvalues and
 * residuals are host arrays of the operator's value type.  Device sums are
 * tree reductions: results agree with the reference's sequential sums to
 * rounding.  Where the reference panics (a subspace of size 0, fewer
 * eigenvalues or eigenvector entries than the requested count) the call
 * returns SX_ERR_COMPUTATION with a message that names the panic. */
typedef struct {
  uint64_t iterations;
  int converged;
  uint64_t num_eigenvalues; /* entries written to eigenvalues */
  uint64_t num_columns;     /* residuals and eigenvector columns */
} sx_eigen_result;
/* PowerIterationOptions (eigen.rs:16-34): 100, 1e-8, normalize */
typedef struct {
  uint64_t max_iter;
  double tol;
  int normalize;
} sx_power_options;
void sx_power_options_default(sx_power_options* o);
/* power_iteration (eigen.rs:124-293): largest eigenvalue by magnitude
 * growth; eigenvector (n entries, may be NULL) and ||A x - lambda x||.
 * DimensionMismatch{expected: n, found: x0_len} for a wrong x0 length. */
int sx_power_iteration(sx_ctx ctx, sx_op a, const sx_power_options* opt, const void* x0, uint64_t x0_len,
                       sx_mem mem, void* eigenvalue, void* eigenvector, void* residual, sx_eigen_result* result);
/* LanczosOptions (eigen.rs:37-61): 1000, 20, 1e-8, 1, eigenvectors */
typedef struct {
  uint64_t max_iter;
  uint64_t max_subspace_size;
  double tol;
  uint64_t num_eigenvalues;
  int compute_eigenvectors;
} sx_lanczos_options;
void sx_lanczos_options_default(sx_lanczos_options* o);
/* lanczos (eigen.rs:295-494, tridiagonal solvers :512-952).  Room needed:
 * eigenvalues and residuals min(num_eigenvalues, subspace) entries,
 * eigenvectors n x that many (row-major, column k = Ritz vector k; may be
 * NULL; ignored without compute_eigenvectors).  The Lanczos basis lives on
 * the device (subspace x n values; max_subspace_size <= 4096). */
int sx_lanczos(sx_ctx ctx, sx_op a, const sx_lanczos_options* opt, const void* v0, uint64_t v0_len, sx_mem mem,
               void* eigenvalues, void* eigenvectors, void* residuals, sx_eigen_result* result);
/* The host tridiagonal eigensolver sx_lanczos runs between its steps
 * (solve_tridiagonal_eigenproblem, eigen.rs:512-952: QL sweeps above three
 * rows, closed forms below), FP64, no device work.  alpha has m entries,
 * beta beta_len (m - 1, else DimensionMismatch).  Room: max(1, min(num, m))
 * values and as many eigenvectors of m entries (vector k at vectors[k m]);
 * count receives the number written.  IterativeSolverFailure when the QL
 * sweep gives up, ValueError for m = 0, as the reference. */
int sx_tridiag_eig(const double* alpha, const double* beta, uint64_t m, uint64_t beta_len, uint64_t num,
                   double* values, double* vectors, uint64_t* count);

/* ------------------------------------------- mixed precision (no reference
 * counterpart; nearest dense analogue scirs2-linalg mixed_precision) */
/* FP32 preconditioned CG inside an FP64 refinement loop.  FP64 holds the
 * solution, the true residual r = b - A x and its norms; every Krylov
 * iteration runs in FP32.  Two outer loops:
 *   SX_IR_REPLACE (default): one FP32 CG run split into segments.  A segment
 *     ends when the FP32 recursive residual has fallen by replace_factor;
 *     then x += x32 (FP64), r = b - A x (FP64) replaces the FP32 residual and
 *     the search direction continues with beta = r.z / r_old.z_old, so the
 *     Krylov progress carries over (residual replacement, "reliable
 *     updates").  outer_iterations counts replacements, max_inner caps each
 *     segment, inner_rtol is unused.
 *   SX_IR_RESTART: classic refinement, x = x0; repeat { r = b - A x (FP64);
 *     solve A d = r/||r|| with FP32 PCG from zero to inner_rtol;
 *     x += ||r|| d (FP64) }.
 * Both stop when ||r||_2 <= tol ||b||_2 (FP64 true residual, converged = 1),
 * and stop unconverged when the FP64 residual stops falling (halving fails
 * twice for REPLACE, once for RESTART): with kappa(A) * 2^-24 near 1 the
 * FP32 iteration cannot help and the caller should fall back to an FP64 solve.
 * a64 must be SX_F64; the FP32 copy is made inside (or pass a32). */
#define SX_IR_REPLACE 0
#define SX_IR_RESTART 1
typedef struct {
  uint64_t max_outer;    /* default 30 */
  uint64_t max_inner;    /* default 10000 (RESTART: per inner solve; REPLACE: per segment) */
  double tol;            /* default 1e-10 */
  double inner_rtol;     /* default 1e-4 (RESTART only) */
  const void* x0;        /* FP64, NULL = zeros */
  sx_op preconditioner;  /* FP32 operator (JACOBI/IC0/FSAI) or NULL = Jacobi of a32 */
  sx_op a32;             /* optional FP32 copy of a64 */
  int mode;              /* SX_IR_REPLACE (default) or SX_IR_RESTART */
  int reserved;
  double replace_factor; /* default 0.1 (REPLACE only): FP32 residual drop per segment */
} sx_ir_options;
typedef struct {
  uint64_t outer_iterations;
  uint64_t inner_iterations;
  double rel_residual;   /* final FP64 true relative residual ||b - A x|| / ||b|| */
  int converged;
} sx_ir_result;
void sx_ir_options_default(sx_ir_options* o);
int sx_cg_mixed(sx_ctx ctx, sx_op a64, const double* b, uint64_t b_len, const sx_ir_options* opt,
                double* x_out, sx_mem mem, sx_ir_result* res);

/* ------------------------------ learned factorised sparse approximate inverse
 * (no reference counterpart; nearest relative SpaiPreconditioner,
 * linalg/spai.rs:15-192, a different method).  A message-passing network
 * over the graph of A predicts a lower-triangular G on the pattern of
 * lower(A) with a softplus diagonal; M^-1 = G G^T is applied as two SpMVs.
 * Trained on the device by its own forward/backward kernels with the
 * random-probe loss ||(G^T A G - I) Z||^2 / (k n) on the Jacobi-scaled A. */
typedef struct sx_gnn_s* sx_gnn;
uint64_t sx_gnn_num_params(void);
/* params: sx_gnn_num_params() floats, or NULL for a seeded initialisation
 * that starts at G = D^-1/2 (Jacobi). */
int sx_gnn_create(sx_ctx ctx, const float* params, uint64_t seed, sx_gnn* out);
int sx_gnn_destroy(sx_gnn net);
int sx_gnn_get_params(sx_ctx ctx, sx_gnn net, float* out);
int sx_gnn_set_params(sx_ctx ctx, sx_gnn net, const float* in);
/* Loss and gradient without an update.  probes: host n x 4 row-major, or
 * NULL for seeded Gaussian probes; grad_out: host, may be NULL. */
int sx_gnn_loss_grad(sx_ctx ctx, sx_gnn net, sx_op a, const float* probes, uint64_t seed,
                     float* loss_out, float* grad_out);
/* One Adam step on the probe loss of a (4 seeded probes). */
int sx_gnn_train_step(sx_ctx ctx, sx_gnn net, sx_op a, uint64_t seed, float lr, float* loss_out);
/* Predicted G^ values in pattern order (each row: strict-lower entries by
 * column, then the diagonal); g_out may be NULL to query the count. */
int sx_gnn_edge_values(sx_ctx ctx, sx_gnn net, sx_op a, float* g_out, uint64_t* ng_out);
/* The preconditioner M^-1 = G G^T for a (same dtype as a). */
int sx_precond_learned(sx_ctx ctx, sx_op a, sx_gnn net, sx_op* out);

/* --------------------------------------------- batched PCG (no reference
 * counterpart: batches the one-system-per-call cg of iterative.rs:40-162) */
/* Thousands of independent SPD systems stored as one block-diagonal CSR
 * (system s owns rows and columns [sys_ptr[s], sys_ptr[s+1])).  Per system:
 * FP64 iterative refinement around an FP32 Jacobi-PCG, stopping when
 * ||b_s - A_s x_s|| <= max(atol, rtol ||b_s||) in FP64.  Each refinement pass
 * runs every active system's FP32 PCG in one persistent launch (a thread
 * block per system, systems taken largest first, per-system exits); the
 * refinement loop with its FP64 residuals, per-system retirement and next
 * queue runs on the device as one CUDA graph.  The launch shape is chosen
 * by the context's autotuner and cached per batch size statistics. */
typedef struct {
  uint64_t max_iter;   /* inner iterations per refinement step, default 10000 */
  double rtol;         /* default 1e-8 (FP64 true residual, per system) */
  double atol;         /* default 0 */
  double inner_rtol;   /* default 1e-4 */
  uint64_t max_outer;  /* default 30 */
} sx_batched_options;
typedef struct {
  uint64_t inner_iterations;
  double rel_residual; /* final FP64 true relative residual of the system */
  int converged;
} sx_batched_result;
typedef struct {
  uint64_t outer_iterations;
  uint64_t converged_systems;
  uint64_t max_inner_iterations;
  uint64_t total_inner_iterations;
  double worst_rel_residual;
  uint64_t kernel_launches;
  uint32_t threads_per_block; /* launch shape the autotuner chose for the */
  uint32_t blocks_per_sm;     /* persistent per-system kernel             */
} sx_batched_summary;
void sx_batched_options_default(sx_batched_options* o);
/* a64: FP64 block-diagonal CSR; a32: its FP32 copy (NULL = made inside);
 * per_system: nsys entries or NULL. */
int sx_batched_pcg(sx_ctx ctx, sx_op a64, sx_op a32, const int64_t* sys_ptr, uint64_t nsys,
                   const double* b, double* x, const sx_batched_options* opt, sx_mem mem,
                   sx_batched_result* per_system, sx_batched_summary* summary);

/* FP64 true relative residual ||b - A x||_2 / ||b||_2 of an FP64 CSR. */
int sx_true_rel_residual(sx_ctx ctx, sx_op a64, const double* b, const double* x, sx_mem mem,
                         double* out);

/* The same residual for callers that cannot allocate device memory while
 * they run (a framework that owns all GPU memory through its own pool, a
 * real-time loop that must not stall on an allocation).  No counterpart in
 * the reference.  b and x are device pointers; nothing is allocated: the
 * reduction scratch is a file-scope device array of 1,572,912 bytes (about
 * 1.5 MiB) that every GPU which loads the library holds until exit.  At most 16,777,216 rows
 * (SX_ERR_VALUE beyond).  Calls share that array, so calls that overlap on
 * the GPU race and must be serialised by the caller.  The first call on a
 * device looks the array up (cudaGetSymbolAddress); make it before any
 * stream capture.  The residual entries b - A x are bit-identical to those
 * of sx_true_rel_residual; the two norms are summed in a different order, so
 * the returned ratio agrees with it to the rounding of that order (within
 * 1e-14 relative in the tests), not bit for bit. */
int sx_true_rel_residual_noalloc(sx_ctx ctx, sx_op a64, const double* b_dev, const double* x_dev,
                                 double* out);

#ifdef __cplusplus
}
#endif
#endif /* SCIRS_SPARSE_H */
