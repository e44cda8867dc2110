/* CPU oracle for the scirs2-sparse iterative-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a C++ restatement of the reference's
 * Rust code (scirs2-sparse 0.1.0-alpha.6), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * The product library never links, loads or calls it.
 *
 * Arithmetic rules that make it a faithful restatement:
 *   - compiled with -O2 -ffp-contract=off (Rust never fuses mul+add);
 *   - every sum is a strict left fold starting at zero, in storage order;
 *   - sort_by_key is std::stable_sort on the same key;
 *   - the same epsilon thresholds (F::epsilon() * 10), messages and
 *     iteration counting as the Rust source.
 * Indices are uint64_t (Rust usize).  All pointers are host pointers.
 */
#ifndef SX_ORACLE_H
#define SX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error record: code follows SparseError's declaration order
 * (scirs2-sparse/src/error.rs:9-74), 0 = Ok. */
typedef struct {
  int code;
  uint64_t v0, v1, v2, v3; /* payload: expected/found, index(r,c)/shape(r,c) */
  char msg[256];
} or_err;

typedef struct {
  uint64_t iterations;
  double residual_norm;
  int converged;
  int message; /* same numbering as the device library's sx_message */
} or_result;

/* ---- construction (f32 / f64 variants) ---- */
int or_csr_matrix_new_f64(const double* data, const uint64_t* rows, const uint64_t* cols,
                          uint64_t nnz, uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                          uint64_t* indices_out, double* data_out, or_err* err);
int or_csr_matrix_new_f32(const float* data, const uint64_t* rows, const uint64_t* cols,
                          uint64_t nnz, uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                          uint64_t* indices_out, float* data_out, or_err* err);
int or_csr_matrix_from_raw_check(const uint64_t* indptr, uint64_t indptr_len,
                                 const uint64_t* indices, uint64_t indices_len, uint64_t data_len,
                                 uint64_t nrows, uint64_t ncols, or_err* err);
int or_csr_array_new_check(const uint64_t* indptr, uint64_t indptr_len, const uint64_t* indices,
                           uint64_t indices_len, uint64_t data_len, uint64_t nrows,
                           uint64_t ncols, int* has_sorted_indices, or_err* err);
int or_csr_array_from_triplets_f64(const uint64_t* rows, const uint64_t* cols,
                                   const double* data, uint64_t nnz, uint64_t nrows,
                                   uint64_t ncols, int sorted, uint64_t* indptr_out,
                                   uint64_t* indices_out, double* data_out,
                                   int* has_sorted_indices, or_err* err);
int or_csr_array_from_triplets_f32(const uint64_t* rows, const uint64_t* cols, const float* data,
                                   uint64_t nnz, uint64_t nrows, uint64_t ncols, int sorted,
                                   uint64_t* indptr_out, uint64_t* indices_out, float* data_out,
                                   int* has_sorted_indices, or_err* err);
void or_csr_transpose_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                          uint64_t nrows, uint64_t ncols, uint64_t* indptr_t,
                          uint64_t* indices_t, double* data_t);
void or_csr_transpose_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                          uint64_t nrows, uint64_t ncols, uint64_t* indptr_t,
                          uint64_t* indices_t, float* data_t);
double or_csr_get_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                      uint64_t nrows, uint64_t ncols, uint64_t i, uint64_t j);

/* ---- SpMV ---- */
void or_spmv_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                 uint64_t nrows, const double* x, double* y);
void or_spmv_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                 uint64_t nrows, const float* x, float* y);
/* Same as above with int64 row pointers and int32 columns (generator layout). */
void or_spmv_i32_f64(const int64_t* indptr, const int32_t* indices, const double* data,
                     int64_t nrows, const double* x, double* y);
void or_spmv_i32_f32(const int64_t* indptr, const int32_t* indices, const float* data,
                     int64_t nrows, const float* x, float* y);

/* ---- operators (LinearOperator restatements) ---- */
typedef struct or_op or_op;
or_op* or_op_csr(int f64, const uint64_t* indptr, const uint64_t* indices, const void* data,
                 uint64_t nrows, uint64_t ncols);
or_op* or_op_csr_i32(int f64, const int64_t* indptr, const int32_t* indices, const void* data,
                     int64_t nrows, int64_t ncols);
or_op* or_op_identity(int f64, uint64_t n);
or_op* or_op_scaled_identity(int f64, uint64_t n, double scale);
or_op* or_op_diagonal(int f64, const void* diag, uint64_t n);
/* JacobiPreconditioner::new from a CSR operator; NULL + err on a zero diagonal. */
or_op* or_op_jacobi(const or_op* csr, or_err* err);
or_op* or_op_jacobi_from_diagonal(int f64, const void* diag, uint64_t n, or_err* err);
/* IC0Preconditioner::new; fast=1 applies the backward solve through a
 * transposed factor in the same subtraction order (bit-identical). */
or_op* or_op_ic0(const or_op* csr, int fast, or_err* err);
/* Factorised approximate inverse M^-1 = G G^T from a lower-triangular CSR G. */
or_op* or_op_fsai(const or_op* g_csr);
void or_op_destroy(or_op* op);
int or_op_matvec(const or_op* op, const void* x, void* y);
uint64_t or_op_rows(const or_op* op);
/* IC(0) factor export: nnz of L and its arrays. */
uint64_t or_ic0_nnz(const or_op* ic0);
void or_ic0_factor(const or_op* ic0, uint64_t* indptr, uint64_t* indices, void* data);

/* ---- solvers (iterative.rs) ---- */
int or_cg(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
          const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err);
int or_bicgstab(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
                const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
                or_err* err);
int or_gmres(const or_op* a, const void* b, uint64_t max_iter, uint64_t restart, double rtol,
             double atol, const void* x0, const or_op* m, void* x_out, or_result* res,
             or_err* err);

/* ---- FP64 iterative refinement around an FP32 inner PCG (no reference
 * counterpart; restates the device algorithm of the same name) ---- */
typedef struct {
  uint64_t max_outer;
  uint64_t max_inner;
  double tol;        /* outer stop: ||b - A x||_2 <= tol * ||b||_2, FP64 */
  double inner_rtol; /* inner FP32 PCG relative tolerance */
  int jacobi;        /* 1: Jacobi inner preconditioner, 0: none */
} or_ir_options;
typedef struct {
  uint64_t outer_iterations;
  uint64_t inner_iterations;
  double rel_residual; /* final FP64 true relative residual */
  int converged;
} or_ir_result;
int or_cg_mixed_ir(const int64_t* indptr, const int32_t* indices, const double* data, int64_t n,
                   const double* b, const or_ir_options* opt, double* x, or_ir_result* res);
/* FP32 PCG with FP64 residual replacement every time the FP32 residual has
 * fallen by delta (restates sx_cg_mixed, mode SX_IR_REPLACE). */
int or_cg_mixed_replace(const int64_t* indptr, const int32_t* indices, const double* data, int64_t n,
                        const double* b, const or_ir_options* opt, double delta, double* x,
                        or_ir_result* res);

/* ---- bicg (iterative.rs:189-345), cgs (cgs.rs:15-193), qmr (qmr.rs:44-259),
 * minres (minres.rs:66-257), lgmres (lgmres.rs:58-327) ---- */
int or_bicg(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
            const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
            or_err* err);
int or_cgs(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
           const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err);
int or_qmr(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
           const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
           or_err* err);
int or_minres(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
              const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err);
int or_lgmres(const or_op* a, const void* b, uint64_t max_iter, uint64_t inner_m, double rtol,
              double atol, const void* x0, const or_op* m, void* x_out, or_result* res,
              or_err* err);

/* ILU0Preconditioner::new (preconditioners.rs:209-324) and SSORPreconditioner::new
 * (:103-131) on a CSR operator; NULL with err set on failure.  The SSOR
 * operator refers to the CSR operator, which must outlive it. */
or_op* or_op_ilu0(const or_op* a, or_err* err);
or_op* or_op_ssor(const or_op* a, double omega, or_err* err);
/* FP64 true relative residual ||b - A x|| / ||b|| with sequential sums. */
double or_true_rel_residual(const int64_t* indptr, const int32_t* indices, const double* data,
                            int64_t n, const double* b, const double* x);

/* ---- symmetric CSR, lower triangle stored (sym_csr.rs, sym_ops.rs) ---- */
/* SymCsrMatrix::new validation (sym_csr.rs:64-134); 0 = Ok.  A decreasing
 * or overrunning indptr (a slice panic in Rust) is InconsistentData. */
int or_sym_csr_check(uint64_t data_len, const uint64_t* indptr, uint64_t indptr_len,
                     const uint64_t* indices, uint64_t nnz, uint64_t nrows, uint64_t ncols,
                     or_err* err);
/* sym_csr_matvec (sym_ops.rs:56-90). */
void or_sym_csr_matvec_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                           uint64_t n, const double* x, double* y);
void or_sym_csr_matvec_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                           uint64_t n, const float* x, float* y);
/* SymCsrMatrix::nnz (sym_csr.rs:254-268), get (sym_csr.rs:280-298). */
uint64_t or_sym_csr_nnz(const uint64_t* indptr, const uint64_t* indices, uint64_t nnz_stored,
                        uint64_t n);
double or_sym_csr_get_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                          uint64_t n, uint64_t row, uint64_t col);
/* sym_csr_trace (sym_ops.rs:317-335), sym_csr_quadratic_form (:271-283). */
double or_sym_csr_trace_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                            uint64_t n);
float or_sym_csr_trace_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                           uint64_t n);
double or_sym_csr_quadratic_form_f64(const uint64_t* indptr, const uint64_t* indices,
                                     const double* data, uint64_t n, const double* x);
float or_sym_csr_quadratic_form_f32(const uint64_t* indptr, const uint64_t* indices,
                                    const float* data, uint64_t n, const float* x);
/* sym_csr_rank1_update (sym_ops.rs:179-233): returns the new nnz; with
 * indptr_out (n + 1) / indices_out / data_out non-null (room for n(n+1)/2
 * entries) also the new arrays. */
uint64_t or_sym_csr_rank1_update_f64(const uint64_t* indptr, const uint64_t* indices,
                                     const double* data, uint64_t n, const double* x,
                                     double alpha, uint64_t* indptr_out, uint64_t* indices_out,
                                     double* data_out);
uint64_t or_sym_csr_rank1_update_f32(const uint64_t* indptr, const uint64_t* indices,
                                     const float* data, uint64_t n, const float* x, float alpha,
                                     uint64_t* indptr_out, uint64_t* indices_out,
                                     float* data_out);
/* SymCsrMatrix::from_csr (sym_csr.rs:149-225) on CSR arrays: returns 0 and
 * the lower part (room for nnz entries) or an error (ValueError). */
int or_sym_csr_from_csr_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                            uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                            uint64_t* indices_out, double* data_out, or_err* err);
int or_sym_csr_from_csr_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                            uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                            uint64_t* indices_out, float* data_out, or_err* err);

/* ---- eigen (linalg/eigen.rs) ---- */
typedef struct {
  uint64_t iterations;
  int converged;
  uint64_t count; /* eigenvalues returned */
  uint64_t num;   /* min(num_eigenvalues, subspace): residual / vector columns */
} or_eig_info;
/* power_iteration (eigen.rs:124-293) on a SymCsrMatrix's arrays; x0 may be
 * NULL (then e_0); vec: n entries. */
int or_power_iteration_f64(const uint64_t* indptr, const uint64_t* indices, const double* data, uint64_t n,
                           uint64_t max_iter, double tol, int normalize, const double* x0, uint64_t x0_len,
                           double* lambda, double* vec, double* resid, or_eig_info* info, or_err* err);
int or_power_iteration_f32(const uint64_t* indptr, const uint64_t* indices, const float* data, uint64_t n,
                           uint64_t max_iter, double tol, int normalize, const float* x0, uint64_t x0_len,
                           float* lambda, float* vec, float* resid, or_eig_info* info, or_err* err);
/* lanczos (eigen.rs:295-494): vals and resids have room for num_eigenvalues,
 * vecs for n * num (row-major, column k = Ritz vector k) when compute_vecs. */
int or_lanczos_f64(const uint64_t* indptr, const uint64_t* indices, const double* data, uint64_t n,
                   uint64_t max_iter, uint64_t max_subspace, double tol, uint64_t num_eigenvalues, int compute_vecs,
                   const double* v0, uint64_t v0_len, double* vals, double* vecs, double* resids, or_eig_info* info,
                   or_err* err);
int or_lanczos_f32(const uint64_t* indptr, const uint64_t* indices, const float* data, uint64_t n, uint64_t max_iter,
                   uint64_t max_subspace, double tol, uint64_t num_eigenvalues, int compute_vecs, const float* v0,
                   uint64_t v0_len, float* vals, float* vecs, float* resids, or_eig_info* info, or_err* err);
/* solve_tridiagonal_eigenproblem (eigen.rs:512-646): vecs (count x m) holds
 * eigenvector k at vecs[k * m .. k * m + m). */
int or_tridiag_eig_f64(const double* alpha, const double* beta, uint64_t m, uint64_t beta_len, uint64_t num,
                       double* vals, double* vecs, uint64_t* count, or_err* err);
/* solve_cubic (eigen.rs:890-952): returns the number of roots written. */
uint64_t or_solve_cubic_f64(double p, double q, double r, double* roots);

/* ---- host threads ----
 * Row-parallel SpMV and elementwise vector loops may use several host
 * threads; every row sum and element update keeps its arithmetic, so results
 * are bit-identical to one thread (the default).  Reductions stay serial. */
void or_set_threads(int n);
int or_get_threads(void);

/* ---- workload generators (sx_gen_oracle.cpp) ----
 * Restatement of the library's seeded generators (kind numbering of
 * sx_gen_kind), bit-identical to them. */
int or_gen_matrix(int kind, int64_t nx, int64_t ny, int64_t nz, uint64_t seed, double p0, double p1,
                  int64_t* n_out, int64_t* nnz_out, int64_t* indptr, int32_t* indices, double* vals);
void or_gen_batch_sides(uint64_t nsys, int64_t side_min, int64_t side_max, uint64_t seed, int64_t* sides);
uint64_t or_gen_batch_system_seed(uint64_t seed, uint64_t s);
void or_gen_rhs_normal(uint64_t seed, int64_t n, double* b);

#ifdef __cplusplus
}
#endif
#endif
