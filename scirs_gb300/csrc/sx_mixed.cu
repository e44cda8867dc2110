// Mixed precision: FP64 refinement around an FP32 preconditioned CG (no
// reference counterpart; the nearest relative is the dense scirs2-linalg
// mixed_precision module).  FP64 is used only for the true residual
// r = b - A x, its norm, and the solution accumulation; every inner
// iteration runs in FP32.  This file holds the entry point, the restart
// loop and the FP64 true residual; the residual-replacement loop shares the
// CG kernels and graphs of sx_krylov.cu and lives there.
//
// restart loop:
//   x = x0;  loop: r = b - A x (FP64);  stop if ||r|| <= tol ||b||;
//            solve A d = r / ||r|| with FP32 PCG to inner_rtol;
//            x += ||r|| d  (FP64)

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "sx_mixed.cuh"

namespace sx {

struct ScaleDown {
  const double* r;
  float* r32;
  const IrNorms* nrm;
  static constexpr bool kReduce = false;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<double>&) const {
    r32[i] = (float)(r[i] * nrm->inv_rnorm);
  }
  __device__ void finish(const Acc3<double>&) const {}
};

struct Accumulate {
  double* x;
  const float* d;
  const IrNorms* nrm;
  static constexpr bool kReduce = false;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<double>&) const {
    x[i] = x[i] + nrm->rnorm * (double)d[i];
  }
  __device__ void finish(const Acc3<double>&) const {}
};

}  // namespace sx

using namespace sx;

extern "C" {

void sx_ir_options_default(sx_ir_options* o) {
  o->max_outer = 30;
  o->max_inner = 10000;
  o->tol = 1e-10;
  o->inner_rtol = 1e-4;
  o->x0 = nullptr;
  o->preconditioner = nullptr;
  o->a32 = nullptr;
  o->mode = SX_IR_REPLACE;
  o->reserved = 0;
  o->replace_factor = 0.1;
}

int sx_true_rel_residual(sx_ctx ctx, sx_op a64, const double* b, const double* x, sx_mem mem,
                         double* out) {
  if (!ctx || !a64 || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a64->kind != SX_OP_CSR || a64->dtype != SX_F64)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: needs an FP64 CSR matrix");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a64->nrows;
  double *db = nullptr, *dx = nullptr, *dr = nullptr;
  IrNorms* nrm = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&dr, std::max<int64_t>(n, 1) * 8))) break;
    if ((rc = dev_alloc((void**)&nrm, sizeof(IrNorms)))) break;
    if (mem == SX_MEM_DEVICE) {
      db = (double*)b;
      dx = (double*)x;
    } else {
      if ((rc = dev_alloc((void**)&db, std::max<int64_t>(n, 1) * 8))) break;
      if ((rc = dev_alloc((void**)&dx, std::max<int64_t>(a64->ncols, 1) * 8))) break;
      cudaMemcpyAsync(db, b, n * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(dx, x, a64->ncols * 8, cudaMemcpyHostToDevice, ctx->stream);
    }
    cudaMemsetAsync(nrm, 0, sizeof(IrNorms), ctx->stream);
    if ((rc = launch_csr<double>(ctx, a64->csr, dx, dr, EpiIrResid{db, nrm}))) break;
    IrNorms h{0, 0, 0, 0};
    cudaMemcpyAsync(&h, nrm, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "true residual", __FILE__, __LINE__); break; }
    *out = std::sqrt(h.rr) / std::sqrt(h.bb);
  } while (0);
  dev_free(dr);
  dev_free(nrm);
  if (mem != SX_MEM_DEVICE) {
    dev_free(db);
    dev_free(dx);
  }
  return rc == SX_OK ? clear_error() : rc;
}

int sx_cg_mixed(sx_ctx ctx, sx_op a64, const double* b, uint64_t b_len, const sx_ir_options* opt,
                double* x_out, sx_mem mem, sx_ir_result* res) {
  if (!ctx || !a64) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a64->kind != SX_OP_CSR || a64->dtype != SX_F64)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: needs an FP64 CSR matrix");
  if (a64->nrows != a64->ncols)
    return set_error(SX_ERR_VALUE, "Value error: Matrix must be square for CG solver");
  if (b_len != (uint64_t)a64->nrows)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a64->nrows) + ", found " +
                         std::to_string(b_len),
                     (uint64_t)a64->nrows, b_len);
  sx_ir_options d;
  if (!opt) { sx_ir_options_default(&d); opt = &d; }
  if (opt->mode != SX_IR_REPLACE && opt->mode != SX_IR_RESTART)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: mixed-precision mode");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a64->nrows;
  sx_op a32 = opt->a32, own32 = nullptr, m = opt->preconditioner, ownm = nullptr;
  int rc = SX_OK;
  double *db = nullptr, *dx = nullptr, *dr = nullptr;
  float *r32 = nullptr, *d32 = nullptr;
  IrNorms* nrm = nullptr;
  uint64_t outer = 0, inner = 0;
  double rel = 0.0;
  int converged = 0;
  do {
    if (!a32) {
      if ((rc = sx_csr_astype(ctx, a64, SX_F32, &own32))) break;
      a32 = own32;
    }
    if (!m) {
      if ((rc = sx_precond_jacobi(ctx, a32, &ownm))) break;
      m = ownm;
    }
    const size_t nb = std::max<int64_t>(n, 1);
    if ((rc = dev_alloc((void**)&db, nb * 8))) break;
    if ((rc = dev_alloc((void**)&dx, nb * 8))) break;
    if ((rc = dev_alloc((void**)&dr, nb * 8))) break;
    if ((rc = dev_alloc((void**)&r32, nb * 4))) break;
    if ((rc = dev_alloc((void**)&d32, nb * 4))) break;
    if ((rc = dev_alloc((void**)&nrm, sizeof(IrNorms)))) break;
    const cudaMemcpyKind kin = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyAsync(db, b, n * 8, kin, ctx->stream);
    if (opt->x0) cudaMemcpyAsync(dx, opt->x0, n * 8, kin, ctx->stream);
    else cudaMemsetAsync(dx, 0, n * 8, ctx->stream);
    if (opt->mode != SX_IR_RESTART) {
      rc = cg_mixed_replace(ctx, a64, a32, m, db, dx, dr, nrm, opt, &outer, &inner, &rel, &converged);
      if (rc) break;
      const cudaMemcpyKind kout = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
      cudaMemcpyAsync(x_out, dx, n * 8, kout, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "solution copy", __FILE__, __LINE__);
      break;
    }
    sx_cg_options io;
    sx_cg_options_default(&io);
    io.max_iter = opt->max_inner;
    io.rtol = opt->inner_rtol;
    io.atol = 0.0;
    io.preconditioner = m;
    while (true) {
      // refinement residual: FMA row sums (a few ulp per row, half the FP64 work)
      if ((rc = launch_csr<double, EpiIrResid, true>(ctx, a64->csr, dx, dr, EpiIrResid{db, nrm}))) break;
      IrNorms h{0, 0, 0, 0};
      cudaMemcpyAsync(&h, nrm, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "refinement residual", __FILE__, __LINE__); break; }
      const double rnorm = std::sqrt(h.rr), bnorm = std::sqrt(h.bb);
      const double prev = rel;
      rel = bnorm > 0 ? rnorm / bnorm : rnorm;
      if (rnorm <= opt->tol * bnorm) { converged = 1; break; }
      if (outer >= opt->max_outer) break;
      // stagnation: an FP32 correction that no longer halves the FP64
      // residual (kappa(A) * eps_fp32 is near 1) ends the refinement
      if (outer > 0 && !(rel < 0.5 * prev)) break;
      if ((rc = launch_vec<double>(ctx, n, ScaleDown{dr, r32, nrm}))) break;
      sx_iter_result ir;
      if ((rc = sx_cg(ctx, a32, r32, (uint64_t)n, &io, d32, SX_MEM_DEVICE, &ir))) break;
      inner += ir.iterations;
      if ((rc = launch_vec<double>(ctx, n, Accumulate{dx, d32, nrm}))) break;
      ++outer;
    }
    if (rc) break;
    const cudaMemcpyKind kout = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaMemcpyAsync(x_out, dx, n * 8, kout, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "solution copy", __FILE__, __LINE__);
  } while (0);
  dev_free(db); dev_free(dx); dev_free(dr); dev_free(r32); dev_free(d32); dev_free(nrm);
  if (ownm) destroy_op_internal(ownm);
  if (own32) destroy_op_internal(own32);
  if (rc != SX_OK) return rc;
  if (res) {
    res->outer_iterations = outer;
    res->inner_iterations = inner;
    res->rel_residual = rel;
    res->converged = converged;
  }
  return clear_error();
}

}  // extern "C"
