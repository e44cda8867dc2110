/* scirs_sparse_gen.h -- seeded synthetic workloads for the sparse solve path.
 *
 * No reference counterpart: the reference crate builds its test matrices
 * inline and ships no PDE generators.  These are host functions (no GPU
 * needed), deterministic for a seed and independent of the thread count.
 * Output CSR: int64 row pointers (n + 1), int32 columns sorted within each
 * row without duplicates, FP64 values; natural ordering (x fastest),
 * Dirichlet boundary nodes eliminated.
 */
#ifndef SCIRS_SPARSE_GEN_H
#define SCIRS_SPARSE_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SX_GEN_POISSON2D = 0, /* 5-point 4/-1 on nx x ny */
  SX_GEN_LAPLACE3D = 1, /* 7-point 6/-1 on nx x ny x nz */
  SX_GEN_VARCOEF3D = 2, /* 7-point, cell c = exp(param0 * N(0,1)), harmonic faces */
  SX_GEN_VARCOEF2D = 3, /* 5-point, same coefficients in 2D */
  SX_GEN_ANISO_Q1 = 4,  /* bilinear FEM, K = R(param1) diag(1, 1/param0) R^T, 9-point */
  SX_GEN_POWERLAW = 5   /* n = nx rows, power-law lengths (mean param0, max param1),
                           uniform distinct columns, values U(-1, 1) */
} sx_gen_kind;

typedef struct {
  int kind;
  int64_t nx, ny, nz;
  uint64_t seed;
  double param0, param1;
} sx_gen_spec;

/* Call once with indptr == NULL to get n and nnz, then with buffers of
 * n + 1, nnz and nnz entries.  Returns 0 on success. */
int sx_gen_matrix(const sx_gen_spec* spec, int64_t* n_out, int64_t* nnz_out, int64_t* indptr,
                  int32_t* indices, double* vals);

/* A batch of 2D variable-coefficient 5-point systems (SX_GEN_VARCOEF2D
 * each), square sides uniform in [side_min, side_max], coefficients
 * exp(sigma N(0,1)), assembled as one block-diagonal CSR.  Call with
 * indptr == NULL to get the sizes and sys_ptr (nsys + 1 entries). */
int sx_gen_batch_varcoef2d(uint64_t nsys, int64_t side_min, int64_t side_max, uint64_t seed,
                           double sigma, int64_t* sys_ptr, int64_t* n_out, int64_t* nnz_out,
                           int64_t* indptr, int32_t* indices, double* vals);

/* b_i ~ N(0, 1) from the seed. */
void sx_gen_rhs_normal(uint64_t seed, int64_t n, double* b);

#ifdef __cplusplus
}
#endif
#endif
