// ILU(0) and SSOR preconditioners on the device
// (scirs2-sparse/src/linalg/preconditioners.rs:94-399).
//
// Both are triangular sweeps over the rows of A.  A forward sweep row waits
// on the rows j < i of its pattern, a backward sweep row on the rows j > i;
// rows are handed to warps in dependency-level order with the bounded flag
// waits of the IC(0) solves (sx_sync.cuh).  In a sweep the products of a row
// are gathered by the warp's lanes and lane 0 subtracts them in storage
// order, so every row rounds exactly as the reference's loop does.
//
// ILU(0) factorisation (preconditioners.rs:211-283).  The reference runs
// k = 0..n-1 outermost and, for every later row i that holds column k,
// scales a_ik by the pivot and subtracts its multiple of row k from the
// entries of row i.  Row i thus sees the steps k in ascending order, each
// using row k in its final state.  The device factorises row i in one warp
// (lane 0, the reference's arithmetic in its order) once the rows it
// depends on are final.  The reference finds column k in row i by a scan
// that stops at the first column above k; an entry is therefore used as a
// multiplier only when every column stored before it in the row is smaller
// (for sorted rows: every entry), and those entries come in ascending
// column order, the order of the reference's k loop.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"
#include "sx_sync.cuh"

namespace sx {

struct TriDev {
  DevCsr m;                 // ILU(0): A factorised in place (L below, U on and above the diagonal);
                            // SSOR: a copy of A
  void* div = nullptr;      // ILU(0): last diagonal entry of U per row; SSOR: the diagonal (first entry)
  void* tmp = nullptr;      // forward-sweep result
  int* ready = nullptr;     // 2 n flags (forward, backward)
  int* ctl = nullptr;       // [0] forward counter, [1] backward counter, [2] abort, [3] spare
  int32_t* fwd_order = nullptr;
  int32_t* bwd_order = nullptr;
  double omega = 1.0;       // SSOR
};

void tri_destroy(TriDev* p) {
  if (!p) return;
  dev_free(p->m.indptr);
  dev_free(p->m.indices);
  dev_free(p->m.vals);
  dev_free(p->div);
  dev_free(p->tmp);
  dev_free(p->ready);
  dev_free(p->ctl);
  dev_free(p->fwd_order);
  dev_free(p->bwd_order);
  delete p;
}

int* tri_ctl(sx_op op) { return op && op->tri ? op->tri->ctl : nullptr; }

namespace {

enum : int { E_NONE = 0, E_MISSING_DIAG = 1, E_ZERO_PIVOT = 2 };

// ILU(0) factorisation, one warp per row in forward level order, lane 0
template <typename T>
__global__ void k_ilu0_factor(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, T* val,
                              int64_t n, int* ready, int* ctl, int* err_row, int* err_code,
                              const int32_t* __restrict__ order, unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  const T eps = sizeof(T) == 8 ? (T)2.220446049250313e-16 : (T)1.1920928955078125e-07f;
  while (true) {
    int64_t t = 0;
    if (lane == 0) t = atomicAdd(ctl + 0, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= n) return;
    const int64_t i = order[t];
    if (lane == 0) {
      const int32_t rs = ptr[i], re = ptr[i + 1];
      int32_t run_max = -1;  // largest column stored before the current entry
      for (int32_t p = rs; p < re; ++p) {
        const int32_t k = idx[p];
        const bool found = k > run_max;  // the reference's scan for column k reaches p
        run_max = max(run_max, k);
        if (!found || k >= (int32_t)i) continue;
        if (!wait_flag(ready + k, ctl + 2, wait_ns)) break;
        // pivot: the first diagonal entry of row k (find_diagonal_index)
        int32_t kd = -1;
        for (int32_t q = ptr[k]; q < ptr[k + 1]; ++q)
          if (idx[q] == k) {
            kd = q;
            break;
          }
        const T piv = kd >= 0 ? ldv(val + kd) : T(0);
        const T mult = ldv(val + p) / piv;
        val[p] = mult;
        for (int32_t q = ptr[k]; q < ptr[k + 1]; ++q) {
          const int32_t j = idx[q];
          if (j <= k) continue;
          for (int32_t r = rs; r < re; ++r)
            if (idx[r] == j) {
              val[r] = sub_rn(ldv(val + r), mul_rn(mult, ldv(val + q)));
              break;
            }
        }
      }
      // this row's own checks (preconditioners.rs:215-225 at step k = i)
      int32_t di = -1;
      for (int32_t q = rs; q < re; ++q)
        if (idx[q] == (int32_t)i) {
          di = q;
          break;
        }
      if (di < 0) {
        err_code[i] = E_MISSING_DIAG;
        atomicMin(err_row, (int)i);
      } else if (fabs(ldv(val + di)) < eps) {
        err_code[i] = E_ZERO_PIVOT;
        atomicMin(err_row, (int)i);
      }
      publish(ready + i);
    }
    __syncwarp();
  }
}

// per row: ILU(0) divisor = last diagonal entry (1 if none, as the
// reference's diag_val starts at one); SSOR divisor = first diagonal entry
// (CsrMatrix::get) with the zero-diagonal check
template <typename T>
__global__ void k_tri_div(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                          const T* __restrict__ val, int64_t n, int ssor, T* div, int* err_row) {
  const T eps = sizeof(T) == 8 ? (T)2.220446049250313e-16 : (T)1.1920928955078125e-07f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T d = ssor ? T(0) : T(1);
    for (int32_t q = ptr[i]; q < ptr[i + 1]; ++q)
      if (idx[q] == (int32_t)i) {
        d = val[q];
        if (ssor) break;
      }
    div[i] = d;
    if (ssor && fabs(d) < eps) atomicMin(err_row, (int)i);
  }
}

// One triangular sweep.  LOWER: entries j < i, rows in forward order; else
// j > i, rows in backward order.  For each row:
//   s = in_i (times pre_i when pre is set)
//   s = s - c(a_ij) out_j   for the sweep's entries in storage order,
//       c(a) = a (ILU(0)) or omega * a (SSOR)
//   out_i = s / div_i (when div is set)
template <typename T, bool LOWER>
__global__ void k_tri_sweep(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const T* __restrict__ val, int64_t n, const T* __restrict__ in,
                            const T* __restrict__ pre, const T* __restrict__ div, int use_omega, T omega, T* out,
                            int* ready, int* ctl, int counter, const int32_t* __restrict__ order,
                            unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int64_t t = 0;
    if (lane == 0) t = atomicAdd(ctl + counter, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= n) return;
    const int64_t i = order[t];
    const int32_t rs = ptr[i], re = ptr[i + 1];
    T s = in[i];
    if (pre) s = mul_rn(s, pre[i]);
    for (int32_t base = rs; base < re; base += 32) {
      const int32_t k = base + lane;
      T prod = T(0);
      bool act = false;
      if (k < re) {
        const int32_t j = idx[k];
        if (LOWER ? j < (int32_t)i : j > (int32_t)i) {
          wait_flag(ready + j, ctl + 2, wait_ns);
          const T c = use_omega ? mul_rn(omega, val[k]) : val[k];
          prod = mul_rn(c, ldv(out + j));
          act = true;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, act);
      for (int q = 0; q < 32; ++q) {
        const T pq = __shfl_sync(0xffffffffu, prod, q);
        if (lane == 0 && ((m >> q) & 1u)) s = sub_rn(s, pq);
      }
    }
    if (lane == 0) {
      out[i] = div ? s / div[i] : s;
      publish(ready + i);
    }
    __syncwarp();
  }
}

int sweep_grid(sx_ctx ctx) { return ctx->num_sms * 8; }

template <typename T>
int tri_apply_t(sx_ctx ctx, sx_op op, const T* x, T* y) {
  TriDev* d = op->tri;
  const int64_t n = op->nrows;
  if (n <= 0) return SX_OK;
  SX_CUDA(cudaMemsetAsync(d->ready, 0, 2 * n * sizeof(int), ctx->stream));
  SX_CUDA(cudaMemsetAsync(d->ctl, 0, 2 * sizeof(int), ctx->stream));
  const DevCsr& m = d->m;
  const int g = sweep_grid(ctx);
  const bool ssor = op->kind == SX_OP_SSOR;
  const T om = (T)d->omega;
  const T* div = (const T*)d->div;
  // ILU(0): y = L^-1 x (unit diagonal), then U^-1 y dividing by the last
  // diagonal (preconditioners.rs:338-375).  SSOR: y = (D + wL)^-1 x, then
  // w = (D + wU)^-1 (y * D) (preconditioners.rs:148-187).
  k_tri_sweep<T, true><<<g, kBlock, 0, ctx->stream>>>(m.indptr, m.indices, (const T*)m.vals, n, x, nullptr,
                                                      ssor ? div : nullptr, ssor ? 1 : 0, om, (T*)d->tmp,
                                                      d->ready, d->ctl, 0, d->fwd_order, ctx->wait_ns);
  k_tri_sweep<T, false><<<g, kBlock, 0, ctx->stream>>>(m.indptr, m.indices, (const T*)m.vals, n,
                                                       (const T*)d->tmp, ssor ? div : nullptr, div,
                                                       ssor ? 1 : 0, om, y, d->ready + n, d->ctl, 1,
                                                       d->bwd_order, ctx->wait_ns);
  ctx->launches += 2;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

// copy of A's arrays into a TriDev, the level orders and the work buffers
int tri_prepare(sx_ctx ctx, sx_op a, TriDev* d) {
  const int64_t n = a->nrows;
  const DevCsr& A = a->csr;
  const size_t w = elt_size(a->dtype);
  d->m.nrows = d->m.ncols = n;
  d->m.nnz = A.nnz;
  SX_CHECK(dev_alloc((void**)&d->m.indptr, (size_t)(n + 1) * 4));
  SX_CHECK(dev_alloc((void**)&d->m.indices, (size_t)std::max<int64_t>(A.nnz, 1) * 4));
  SX_CHECK(dev_alloc(&d->m.vals, (size_t)std::max<int64_t>(A.nnz, 1) * w));
  SX_CUDA(cudaMemcpyAsync(d->m.indptr, A.indptr, (n + 1) * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  if (A.nnz > 0) {
    SX_CUDA(cudaMemcpyAsync(d->m.indices, A.indices, A.nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(d->m.vals, A.vals, A.nnz * w, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  SX_CHECK(dev_alloc(&d->div, (size_t)std::max<int64_t>(n, 1) * w));
  SX_CHECK(dev_alloc(&d->tmp, (size_t)std::max<int64_t>(n, 1) * w));
  SX_CHECK(dev_alloc((void**)&d->ready, (size_t)std::max<int64_t>(2 * n, 1) * sizeof(int)));
  SX_CHECK(dev_alloc((void**)&d->ctl, 4 * sizeof(int)));
  SX_CUDA(cudaMemsetAsync(d->ctl, 0, 4 * sizeof(int), ctx->stream));
  SX_CHECK(level_order(ctx, d->m, true, &d->fwd_order));
  SX_CHECK(level_order(ctx, d->m, false, &d->bwd_order));
  return SX_OK;
}

sx_op new_tri_op(sx_ctx ctx, sx_op a, int kind) {
  sx_op op = new sx_op_s();
  op->kind = kind;
  op->dtype = a->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = a->nrows;
  op->serial = next_op_serial();
  op->tri = new TriDev();
  return op;
}

int check_square_csr(sx_op a) {
  if (a->kind != SX_OP_CSR) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: not CSR");
  if (a->nrows != a->ncols)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a->nrows) + ", found " +
                         std::to_string(a->ncols),
                     (uint64_t)a->nrows, (uint64_t)a->ncols);
  if (!a->csr.monotone)
    return set_error(SX_ERR_INCONSISTENT_DATA, "Inconsistent data: row pointers must be non-decreasing");
  return SX_OK;
}

}  // namespace

int tri_apply(sx_ctx ctx, sx_op op, const void* x, void* y) {
  if (op->dtype == SX_F64) return tri_apply_t<double>(ctx, op, (const double*)x, (double*)y);
  return tri_apply_t<float>(ctx, op, (const float*)x, (float*)y);
}

}  // namespace sx

using namespace sx;

extern "C" {

int sx_precond_ilu0(sx_ctx ctx, sx_op a, sx_op* out) {
  if (!ctx || !a || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CHECK(check_square_csr(a));
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a->nrows;
  sx_op op = new_tri_op(ctx, a, SX_OP_ILU0);
  TriDev* d = op->tri;
  int* err = nullptr;
  int rc = tri_prepare(ctx, a, d);
  do {
    if (rc != SX_OK) break;
    if ((rc = dev_alloc((void**)&err, (size_t)(n + 1) * sizeof(int)))) break;
    SX_CUDA(cudaMemsetAsync(err + 1, 0, (size_t)n * sizeof(int), ctx->stream));
    const int big = INT_MAX;
    SX_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    SX_CUDA(cudaMemsetAsync(d->ready, 0, (size_t)n * sizeof(int), ctx->stream));
    SX_CUDA(cudaMemsetAsync(d->ctl, 0, 4 * sizeof(int), ctx->stream));
    if (n > 0) {
      if (a->dtype == SX_F64)
        k_ilu0_factor<double><<<sweep_grid(ctx), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (double*)d->m.vals, n, d->ready, d->ctl, err, err + 1, d->fwd_order, ctx->wait_ns);
      else
        k_ilu0_factor<float><<<sweep_grid(ctx), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (float*)d->m.vals, n, d->ready, d->ctl, err, err + 1, d->fwd_order, ctx->wait_ns);
      ctx->launches++;
    }
    int h[4] = {0, 0, 0, 0};
    int row = INT_MAX;
    SX_CUDA(cudaMemcpyAsync(h, d->ctl, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(&row, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "ILU(0) factorisation", __FILE__, __LINE__);
      break;
    }
    if (h[2]) {
      rc = set_error(SX_ERR_DEVICE_TIMEOUT, "Device timeout: an ILU(0) dependency wait exceeded its time limit");
      break;
    }
    if (row != INT_MAX) {
      int code = 0;
      SX_CUDA(cudaMemcpy(&code, err + 1 + row, sizeof(int), cudaMemcpyDeviceToHost));
      rc = set_error(SX_ERR_VALUE, code == E_MISSING_DIAG
                                       ? "Value error: Missing diagonal element at row " + std::to_string(row)
                                       : "Value error: Zero pivot at position " + std::to_string(row));
      break;
    }
    if (n > 0) {
      if (a->dtype == SX_F64)
        k_tri_div<double><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (const double*)d->m.vals, n, 0, (double*)d->div, err);
      else
        k_tri_div<float><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (const float*)d->m.vals, n, 0, (float*)d->div, err);
      ctx->launches++;
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "ILU(0) divisors", __FILE__, __LINE__);
  } while (0);
  dev_free(err);
  if (rc != SX_OK) {
    destroy_op_internal(op);
    return rc;
  }
  *out = op;
  return clear_error();
}

int sx_precond_ssor(sx_ctx ctx, sx_op a, double omega, sx_op* out) {
  if (!ctx || !a || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CHECK(check_square_csr(a));
  *out = nullptr;
  // preconditioners.rs:106-110, compared in the matrix's value type
  const bool bad = a->dtype == SX_F64 ? (omega <= 0.0 || omega >= 2.0)
                                      : ((float)omega <= 0.0f || (float)omega >= 2.0f);
  if (bad) return set_error(SX_ERR_VALUE, "Value error: Relaxation parameter omega must be in (0, 2)");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a->nrows;
  sx_op op = new_tri_op(ctx, a, SX_OP_SSOR);
  TriDev* d = op->tri;
  d->omega = a->dtype == SX_F64 ? omega : (double)(float)omega;
  int* err = nullptr;
  int rc = tri_prepare(ctx, a, d);
  do {
    if (rc != SX_OK) break;
    if ((rc = dev_alloc((void**)&err, sizeof(int) * 4))) break;
    const int big = INT_MAX;
    SX_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (n > 0) {
      if (a->dtype == SX_F64)
        k_tri_div<double><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (const double*)d->m.vals, n, 1, (double*)d->div, err);
      else
        k_tri_div<float><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            d->m.indptr, d->m.indices, (const float*)d->m.vals, n, 1, (float*)d->div, err);
      ctx->launches++;
    }
    int row = INT_MAX;
    SX_CUDA(cudaMemcpyAsync(&row, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "SSOR diagonal", __FILE__, __LINE__);
      break;
    }
    if (row != INT_MAX)
      rc = set_error(SX_ERR_VALUE, "Value error: Zero diagonal element at position " + std::to_string(row));
  } while (0);
  dev_free(err);
  if (rc != SX_OK) {
    destroy_op_internal(op);
    return rc;
  }
  *out = op;
  return clear_error();
}

}  // extern "C"
