// Preconditioners and the multi-kernel operator applies:
//  - JacobiPreconditioner (scirs2-sparse/src/linalg/preconditioners.rs:14-92)
//  - M^-1 = G G^T with an explicit cached G^T (learned factorised SAI)
//  - host-callback operators (a user's dyn LinearOperator)
//  - spmv_device: the plain y = A x used by the ABI's matvec.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cstdio>
#include <string>

#include "sx_launch.cuh"

namespace sx {

int ic0_apply(sx_ctx ctx, sx_op op, const void* x, void* y);  // sx_ic0.cu

int spmv_device(sx_ctx ctx, sx_op a, const void* x, void* y, unsigned flags) {
  if (a->kind == SX_OP_SYM_CSR && (flags & SX_SPMV_SYM_HALF) && !(flags & SX_SPMV_EXACT))
    return sym_half_spmv(ctx, a, x, y);
  // SX_SPMV_EXACT keeps the reference's per-row rounding (bit-exact); without
  // it, FP64 rows are summed with fused multiply-adds (a few ulp per row)
  if (a->dtype == SX_F64) {
    if (flags & SX_SPMV_EXACT)
      return launch_apply<double, EpiPlain<double>, true>(ctx, a, (const double*)x, (double*)y,
                                                          EpiPlain<double>{});
    return launch_apply<double, EpiPlain<double>, false>(ctx, a, (const double*)x, (double*)y,
                                                         EpiPlain<double>{});
  }
  return launch_apply<float, EpiPlain<float>, true>(ctx, a, (const float*)x, (float*)y,
                                                    EpiPlain<float>{});
}

extern "C" int sx_spmv_kernel(sx_ctx ctx, sx_op a, unsigned flags, char* buf, uint64_t len) {
  if (!ctx || !a || !buf || len == 0) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  std::string name;
  const bool exact = (flags & SX_SPMV_EXACT) != 0;
  const int w = (int)elt_size(a->dtype);
  const bool fma = !exact && w == 8;
  switch (a->kind) {
    case SX_OP_CSR: name = spmv_kernel_name(ctx, a->csr, w, fma, false); break;
    case SX_OP_SYM_CSR:
      name = (flags & SX_SPMV_SYM_HALF) && !exact ? std::string("k_sym_half")
                                                  : spmv_kernel_name(ctx, a->csr, w, fma, false);
      break;
    case SX_OP_FSAI:
      name = std::string("G^T: ") + spmv_kernel_name(ctx, a->transpose->csr, w, fma, !exact) +
             "; G: " + spmv_kernel_name(ctx, a->csr, w, fma, !exact);
      break;
    case SX_OP_IC0: name = "k_ic0_forward + k_ic0_backward"; break;
    case SX_OP_ILU0:
    case SX_OP_SSOR: name = "k_tri_sweep (forward) + k_tri_sweep (backward)"; break;
    case SX_OP_HOST: name = "host callback"; break;
    default: name = "k_diag_apply"; break;
  }
  std::snprintf(buf, (size_t)len, "%s", name.c_str());
  return clear_error();
}

int apply_general(sx_ctx ctx, sx_op op, const void* x, void* y) {
  const size_t w = elt_size(op->dtype);
  switch (op->kind) {
    case SX_OP_IC0:
      return ic0_apply(ctx, op, x, y);
    case SX_OP_ILU0:
    case SX_OP_SSOR:
      return tri_apply(ctx, op, x, y);
    case SX_OP_FSAI:
      return spmv_device(ctx, op, x, y, 0);
    case SX_OP_HOST: {
      // stage through host memory and call the user's matvec
      std::vector<char> hx((size_t)op->ncols * w), hy((size_t)op->nrows * w);
      SX_CUDA(cudaMemcpyAsync(hx.data(), x, hx.size(), cudaMemcpyDeviceToHost, ctx->stream));
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      int rc = op->host.fn(op->host.user, hx.data(), hy.data(), (uint64_t)op->ncols);
      if (rc != 0)
        return set_error(SX_ERR_COMPUTATION,
                         "Computation error: host operator returned " + std::to_string(rc));
      SX_CUDA(cudaMemcpyAsync(y, hy.data(), hy.size(), cudaMemcpyHostToDevice, ctx->stream));
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      return SX_OK;
    }
    default:
      return spmv_device(ctx, op, x, y, 0);
  }
}

namespace {

// dinv_i = 1 / get(i, i) with the first duplicate's value (csr.rs:40-44);
// bad = smallest i with |d| < epsilon (preconditioners.rs:29-35).
template <typename T>
__global__ void k_jacobi(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                         const T* __restrict__ vals, int64_t n, T eps, T* dinv,
                         unsigned long long* bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T d = T(0);
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
      if (idx[k] == (int32_t)i) { d = vals[k]; break; }
    if (fabs(d) < eps) atomicMin(bad, (unsigned long long)i);
    dinv[i] = T(1) / d;
  }
}

template <typename T>
__global__ void k_inv_diag(const T* __restrict__ d, int64_t n, T eps, T* dinv,
                           unsigned long long* bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T v = d[i];
    if (fabs(v) < eps) atomicMin(bad, (unsigned long long)i);
    dinv[i] = T(1) / v;
  }
}

}  // namespace
}  // namespace sx

using namespace sx;

static int jacobi_finish(sx_ctx ctx, unsigned long long* d_bad, sx_op op, sx_op* out) {
  unsigned long long hb = ~0ull;
  cudaMemcpyAsync(&hb, d_bad, 8, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  dev_free(d_bad);
  if (e != cudaSuccess) {
    destroy_op_internal(op);
    return cuda_fail(e, "jacobi", __FILE__, __LINE__);
  }
  if (hb != ~0ull) {
    destroy_op_internal(op);
    return set_error(SX_ERR_VALUE,
                     "Value error: Zero diagonal element at position " + std::to_string(hb));
  }
  *out = op;
  return clear_error();
}

extern "C" {

int sx_precond_jacobi(sx_ctx ctx, sx_op a, sx_op* out) {
  if (!ctx || !a || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a->kind != SX_OP_CSR) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: not CSR");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  // JacobiPreconditioner::new walks n = matrix.rows() diagonal positions
  const int64_t n = a->nrows;
  sx_op op = new sx_op_s();
  op->kind = SX_OP_JACOBI;
  op->dtype = a->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = n;
  op->serial = next_op_serial();
  int rc = dev_alloc(&op->diag, std::max<int64_t>(n, 1) * elt_size(a->dtype));
  unsigned long long* bad = nullptr;
  if (rc == SX_OK) rc = dev_alloc((void**)&bad, 8);
  if (rc != SX_OK) { destroy_op_internal(op); return rc; }
  cudaMemsetAsync(bad, 0xff, 8, ctx->stream);
  const int g = vec_grid(ctx, n);
  if (n > 0) {
    if (a->dtype == SX_F64)
      k_jacobi<double><<<g, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices,
                                                      (const double*)a->csr.vals, n,
                                                      2.220446049250313e-16, (double*)op->diag, bad);
    else
      k_jacobi<float><<<g, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices,
                                                     (const float*)a->csr.vals, n,
                                                     1.1920928955078125e-07f, (float*)op->diag, bad);
    ctx->launches++;
  }
  return jacobi_finish(ctx, bad, op, out);
}

int sx_precond_jacobi_from_diagonal(sx_ctx ctx, sx_dtype dtype, const void* diag, uint64_t n,
                                    sx_op* out) {
  if (!ctx || !out || (n > 0 && !diag))
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  const size_t w = elt_size(dtype);
  sx_op op = new sx_op_s();
  op->kind = SX_OP_JACOBI;
  op->dtype = dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = (int64_t)n;
  op->serial = next_op_serial();
  void* d = nullptr;
  unsigned long long* bad = nullptr;
  int rc = dev_alloc(&op->diag, std::max<uint64_t>(n, 1) * w);
  if (rc == SX_OK) rc = dev_alloc(&d, std::max<uint64_t>(n, 1) * w);
  if (rc == SX_OK) rc = dev_alloc((void**)&bad, 8);
  if (rc != SX_OK) { dev_free(d); destroy_op_internal(op); return rc; }
  cudaMemsetAsync(bad, 0xff, 8, ctx->stream);
  if (n > 0) {
    cudaMemcpyAsync(d, diag, n * w, cudaMemcpyHostToDevice, ctx->stream);
    const int g = vec_grid(ctx, (int64_t)n);
    if (dtype == SX_F64)
      k_inv_diag<double><<<g, kBlock, 0, ctx->stream>>>((const double*)d, (int64_t)n,
                                                        2.220446049250313e-16, (double*)op->diag, bad);
    else
      k_inv_diag<float><<<g, kBlock, 0, ctx->stream>>>((const float*)d, (int64_t)n,
                                                       1.1920928955078125e-07f, (float*)op->diag, bad);
    ctx->launches++;
  }
  cudaStreamSynchronize(ctx->stream);
  dev_free(d);
  return jacobi_finish(ctx, bad, op, out);
}

}  // extern "C"

namespace sx {
// FSAI operator that takes over the CSR arrays of g (a temporary the caller
// no longer needs): one transpose for G^T instead of the public entry's
// copy, or none when the caller built G^T (gt, taken over as well).  g's and
// gt's shells are destroyed whatever the outcome.
int fsai_adopt(sx_ctx ctx, sx_op g, sx_op* out, sx_op gt) {
  *out = nullptr;
  sx_op op = new sx_op_s();
  op->kind = SX_OP_FSAI;
  op->dtype = g->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = g->nrows;
  op->serial = next_op_serial();
  int rc = SX_OK;
  if (gt) op->transpose = gt;
  else rc = csr_transpose_internal(ctx, g, &op->transpose);
  if (rc == SX_OK) {
    op->csr = g->csr;
    g->csr = DevCsr();
    rc = dev_alloc(&op->work, std::max<int64_t>(g->nrows, 1) * elt_size(g->dtype));
  }
  destroy_op_internal(g);
  if (rc != SX_OK) { destroy_op_internal(op); return rc; }
  *out = op;
  return SX_OK;
}
}  // namespace sx

extern "C" {

int sx_precond_fsai(sx_ctx ctx, sx_op g, sx_op* out) {
  if (!ctx || !g || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (g->kind != SX_OP_CSR) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: not CSR");
  if (g->nrows != g->ncols) {
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(g->nrows) + ", found " +
                         std::to_string(g->ncols),
                     (uint64_t)g->nrows, (uint64_t)g->ncols);
  }
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  sx_op op = new sx_op_s();
  op->kind = SX_OP_FSAI;
  op->dtype = g->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = g->nrows;
  op->serial = next_op_serial();
  // deep copy of G (the caller keeps its own handle)
  sx_op gt = nullptr;
  int rc = csr_transpose_internal(ctx, g, &gt);
  if (rc != SX_OK) { delete op; return rc; }
  rc = csr_transpose_internal(ctx, gt, &op->transpose);  // (G^T)^T = G, bit-exact
  if (rc != SX_OK) { destroy_op_internal(gt); delete op; return rc; }
  // op->csr = G, op->transpose = G^T
  std::swap(op->csr, op->transpose->csr);
  std::swap(op->transpose->csr, gt->csr);
  destroy_op_internal(gt);
  op->transpose->nrows = op->transpose->ncols = g->nrows;
  rc = dev_alloc(&op->work, std::max<int64_t>(g->nrows, 1) * elt_size(g->dtype));
  if (rc != SX_OK) { destroy_op_internal(op); return rc; }
  *out = op;
  return clear_error();
}

}  // extern "C"
