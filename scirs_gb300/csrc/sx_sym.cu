// Symmetric CSR with lower-triangle storage (scirs2-sparse sym_csr.rs) and the
// operations of sym_ops.rs on it.
//
// sym_csr_matvec (sym_ops.rs:56-90) walks the stored rows once: for entry
// (i, j, v) it adds v x_j to y_i and, off the diagonal, v x_i to y_j.  Entry
// by entry, y_k therefore receives first the terms of its own stored row (in
// storage order) and then, row after row below it, the terms of column k.
// The device keeps that sequence as one merged row per k:
//   row k of C = [stored row k] ++ [row k of (strict lower)^T]
// built with the bit-exact counting-sort transpose (a column's entries in row
// order, storage order within a row).  The exact CSR SpMV of C, which sums
// each row left to right from 0 with separately rounded products, then gives
// the reference's y bit for bit and runs on the tuned CSR kernels (with their
// fused solver epilogues).  get(r, c) on C also matches SymCsrMatrix::get
// (sym_csr.rs:280-298): an upper position's first match lies in the
// transposed part, at the first stored (c, r) of row c.
//
// The stored lower triangle is kept beside C (sym_low) for the accessors,
// to_csr, trace, rank-1 update and the half-storage SpMV, which reads only
// the lower triangle and scatters the transposed terms with atomic adds
// (SX_SPMV_SYM_HALF: fewer bytes, summation order not fixed).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"

namespace sx {
namespace {

int err_value(const std::string& s) { return set_error(SX_ERR_VALUE, "Value error: " + s); }
int err_arg(const char* s) { return set_error(SX_ERR_INVALID_ARGUMENT, std::string("Invalid argument: ") + s); }
int err_dim(uint64_t expected, uint64_t found) {
  return set_error(SX_ERR_DIMENSION_MISMATCH,
                   "Dimension mismatch: expected " + std::to_string(expected) + ", found " + std::to_string(found),
                   expected, found);
}
bool is_sym(sx_op a) { return a && a->kind == SX_OP_SYM_CSR && a->sym_low; }

// ---------------------------------------------------------------- kernels
// rows of the strict lower part (col < row), in storage order
__global__ void k_strict_count(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                               int32_t* cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t c = 0;
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) c += idx[k] < (int32_t)r;
    cnt[r] = c;
  }
}
template <typename T>
__global__ void k_strict_copy(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const T* __restrict__ val, int64_t n, const int32_t* __restrict__ sp, int32_t* si,
                              T* sv) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t o = sp[r];
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k)
      if (idx[k] < (int32_t)r) {
        si[o] = idx[k];
        sv[o] = val[k];
        ++o;
      }
  }
}
// row k of C = stored row k ++ row k of (strict lower)^T
__global__ void k_merge_count(const int32_t* __restrict__ lp, const int32_t* __restrict__ tp, int64_t n,
                              int32_t* cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride)
    cnt[r] = (lp[r + 1] - lp[r]) + (tp[r + 1] - tp[r]);
}
template <typename T>
__global__ void k_merge_copy(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                             const T* __restrict__ lv, const int32_t* __restrict__ tp,
                             const int32_t* __restrict__ ti, const T* __restrict__ tv, int64_t n,
                             const int32_t* __restrict__ cp, int32_t* ci, T* cv) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t o = cp[r];
    for (int32_t k = lp[r]; k < lp[r + 1]; ++k, ++o) {
      ci[o] = li[k];
      cv[o] = lv[k];
    }
    for (int32_t k = tp[r]; k < tp[r + 1]; ++k, ++o) {
      ci[o] = ti[k];
      cv[o] = tv[k];
    }
  }
}

// SymCsrMatrix::is_symmetric (sym_csr.rs:197-225): every stored (i, j, v)
// against get(j, i) (first match in row j, csr.rs:33-48), |v - a_ji| > tol
// means not symmetric (a NaN difference passes, as in the reference)
template <typename T>
__global__ void k_sym_check(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const T* __restrict__ val, int64_t n, T tol, int* bad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int32_t j = idx[k];
      T t = T(0);
      for (int32_t q = ptr[j]; q < ptr[j + 1]; ++q)
        if (idx[q] == (int32_t)i) {
          t = val[q];
          break;
        }
      const T d = fabs(sub_rn(val[k], t));
      if (d > tol) *bad = 1;
    }
  }
}
// the lower part (col <= row) of a CSR matrix in storage order (sym_csr.rs:166-182)
__global__ void k_lower_count(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                              int32_t* cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t c = 0;
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) c += idx[k] <= (int32_t)r;
    cnt[r] = c;
  }
}
template <typename T>
__global__ void k_lower_copy(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const T* __restrict__ val, int64_t n, const int32_t* __restrict__ lp, int32_t* li,
                             T* lv) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t o = lp[r];
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k)
      if (idx[k] <= (int32_t)r) {
        li[o] = idx[k];
        lv[o] = val[k];
        ++o;
      }
  }
}

// first diagonal entry of every row (sym_csr_trace, sym_ops.rs:317-335);
// has[i] = 1 when row i stores its diagonal (SymCsrMatrix::nnz, sym_csr.rs:254-268)
template <typename T>
__global__ void k_first_diag(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const T* __restrict__ val, int64_t n, T* d, int32_t* has) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T v = T(0);
    int32_t h = 0;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
      if (idx[k] == (int32_t)i) {
        v = val[k];
        h = 1;
        break;
      }
    d[i] = v;
    has[i] = h;
  }
}

// Sums in the reference's sequential order (one thread: r = r + a_i, or
// r = r + x_i * y_i with separately rounded products).  Used for the trace
// and the quadratic form, whose results the reference defines by that order.
template <typename T>
__global__ void k_seq_sum(const T* __restrict__ a, const T* __restrict__ b, int64_t n, T* out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  T r = T(0);
  if (b) {
    for (int64_t i = 0; i < n; ++i) r = add_rn(r, mul_rn(a[i], b[i]));
  } else {
    for (int64_t i = 0; i < n; ++i) r = add_rn(r, a[i]);
  }
  *out = r;
}

// sym_csr_rank1_update (sym_ops.rs:179-233): the lower triangle of
// to_dense() (the last stored duplicate of a position wins), plus
// (alpha x_i) x_j, kept where the sum is not zero.  One block per row; the
// count pass and the write pass evaluate the same expression.
template <typename T>
__device__ __forceinline__ T rank1_value(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                         const T* __restrict__ val, int64_t i, int64_t j, T ax_i,
                                         const T* __restrict__ x) {
  T d = T(0);
  for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
    if (idx[k] == (int32_t)j) d = val[k];
  return add_rn(d, mul_rn(ax_i, x[j]));
}
template <typename T>
__global__ void k_rank1_count(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const T* __restrict__ val, int64_t n, const T* __restrict__ x, T alpha,
                              int32_t* cnt) {
  __shared__ int32_t warp_cnt[32];
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const T ax = mul_rn(alpha, x[i]);
    int32_t c = 0;
    for (int64_t j = threadIdx.x; j <= i; j += blockDim.x) c += rank1_value(ptr, idx, val, i, j, ax, x) != T(0);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      int32_t s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += warp_cnt[w];
      cnt[i] = s;
    }
    __syncthreads();
  }
}
template <typename T>
__global__ void k_rank1_write(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const T* __restrict__ val, int64_t n, const T* __restrict__ x, T alpha,
                              const int32_t* __restrict__ np, int32_t* ni, T* nv) {
  __shared__ int32_t warp_cnt[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const T ax = mul_rn(alpha, x[i]);
    int32_t base = np[i];
    // tiles of blockDim.x columns, compacted in column order
    for (int64_t j0 = 0; j0 <= i; j0 += blockDim.x) {
      const int64_t j = j0 + threadIdx.x;
      T v = T(0);
      bool keep = false;
      if (j <= i) {
        v = rank1_value(ptr, idx, val, i, j, ax, x);
        keep = v != T(0);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warp_cnt[wid] = __popc(m);
      __syncthreads();
      int32_t off = base, tot = 0;
      for (int w = 0; w < nw; ++w) {
        if (w < wid) off += warp_cnt[w];
        tot += warp_cnt[w];
      }
      if (keep) {
        const int32_t o = off + __popc(m & ((1u << lane) - 1u));
        ni[o] = (int32_t)j;
        nv[o] = v;
      }
      base += tot;
      __syncthreads();
    }
  }
}

// Half-storage product: each stored entry read once, y_i's own row summed in
// registers, the transposed terms added to y_j atomically.  y starts at 0.
template <typename T>
__global__ void k_sym_half(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const T* __restrict__ val, int64_t n, const T* __restrict__ x, T* y) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T xi = __ldg(x + i);
    T acc = T(0);
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int32_t j = __ldg(idx + k);
      const T v = __ldg(val + k);
      acc = fma(v, __ldg(x + j), acc);
      if (j != (int32_t)i) atomicAdd(y + j, v * xi);
    }
    atomicAdd(y + i, acc);
  }
}

// ------------------------------------------------------------ host helpers
// A device CSR op owning the given arrays (indptr of n + 1 entries).
sx_op wrap_csr(sx_ctx ctx, int dtype, int64_t n, int64_t nnz, int32_t* ptr, int32_t* idx, void* val) {
  sx_op s = new sx_op_s();
  s->kind = SX_OP_CSR;
  s->dtype = dtype;
  s->device = ctx->device;
  s->nrows = s->ncols = n;
  s->serial = next_op_serial();
  s->csr.nrows = s->csr.ncols = n;
  s->csr.nnz = nnz;
  s->csr.indptr = ptr;
  s->csr.indices = idx;
  s->csr.vals = val;
  return s;
}

int sync_check(sx_ctx ctx, const char* what) {
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, what, __FILE__, __LINE__);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what, __FILE__, __LINE__);
  return SX_OK;
}

// Builds C (merged rows) from the lower triangle L into `out`.
template <typename T>
int build_merged(sx_ctx ctx, sx_op low, DevCsr& C) {
  const DevCsr& L = low->csr;
  const int64_t n = L.nrows;
  const int g = vec_grid(ctx, std::max<int64_t>(n, 1));
  const size_t nb = (size_t)std::max<int64_t>(n, 1);
  int32_t *scnt = nullptr, *sp = nullptr, *si = nullptr, *ccnt = nullptr;
  T* sv = nullptr;
  sx_op s = nullptr, st = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&scnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&sp, (nb + 1) * 4))) break;
    if (n > 0) {
      k_strict_count<<<g, kBlock, 0, ctx->stream>>>(L.indptr, L.indices, n, scnt);
      ctx->launches++;
    }
    if ((rc = exclusive_scan_i32(ctx, scnt, n, sp))) break;
    int32_t snnz = 0;
    SX_CUDA(cudaMemcpyAsync(&snnz, sp + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = sync_check(ctx, "symmetric strict count"))) break;
    if ((rc = dev_alloc((void**)&si, (size_t)std::max<int32_t>(snnz, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&sv, (size_t)std::max<int32_t>(snnz, 1) * sizeof(T)))) break;
    if (n > 0) {
      k_strict_copy<T><<<g, kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, n, sp, si, sv);
      ctx->launches++;
    }
    s = wrap_csr(ctx, low->dtype, n, snnz, sp, si, sv);
    sp = nullptr;
    si = nullptr;
    sv = nullptr;
    if ((rc = csr_transpose_internal(ctx, s, &st))) break;
    const DevCsr& Tt = st->csr;
    if ((rc = dev_alloc((void**)&ccnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&C.indptr, (nb + 1) * 4))) break;
    if (n > 0) {
      k_merge_count<<<g, kBlock, 0, ctx->stream>>>(L.indptr, Tt.indptr, n, ccnt);
      ctx->launches++;
    }
    if ((rc = exclusive_scan_i32(ctx, ccnt, n, C.indptr))) break;
    const int64_t cnnz = L.nnz + Tt.nnz;
    C.nrows = C.ncols = n;
    C.nnz = cnnz;
    if ((rc = dev_alloc((void**)&C.indices, (size_t)std::max<int64_t>(cnnz, 1) * 4))) break;
    if ((rc = dev_alloc(&C.vals, (size_t)std::max<int64_t>(cnnz, 1) * sizeof(T)))) break;
    if (n > 0) {
      k_merge_copy<T><<<g, kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, Tt.indptr,
                                                      Tt.indices, (const T*)Tt.vals, n, C.indptr, C.indices,
                                                      (T*)C.vals);
      ctx->launches++;
    }
    if ((rc = sync_check(ctx, "symmetric merge"))) break;
    rc = csr_finalize_stats(ctx, C, (int)sizeof(T));
  } while (0);
  if (s) destroy_op_internal(s);
  if (st) destroy_op_internal(st);
  dev_free(scnt);
  dev_free(sp);
  dev_free(si);
  dev_free(sv);
  dev_free(ccnt);
  return rc;
}

// A symmetric operator over the lower triangle `low` (taken over).
int make_sym(sx_ctx ctx, sx_op low, sx_op* out) {
  sx_op op = new sx_op_s();
  op->kind = SX_OP_SYM_CSR;
  op->dtype = low->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = low->nrows;
  op->serial = next_op_serial();
  op->sym_low = low;
  const int rc = low->dtype == SX_F64 ? build_merged<double>(ctx, low, op->csr) : build_merged<float>(ctx, low, op->csr);
  if (rc != SX_OK) {
    destroy_op_internal(op);
    return rc;
  }
  *out = op;
  return SX_OK;
}

// Replaces op's lower triangle (and C) by `low`; op keeps its handle.
int replace_low(sx_ctx ctx, sx_op op, sx_op low) {
  sx_op fresh = nullptr;
  SX_CHECK(make_sym(ctx, low, &fresh));
  std::swap(op->csr, fresh->csr);
  std::swap(op->sym_low, fresh->sym_low);
  op->serial = fresh->serial;  // new buffers: never replay a graph of the old ones
  destroy_op_internal(fresh);
  return SX_OK;
}

template <typename T>
int first_diag(sx_ctx ctx, const DevCsr& L, T** d, int32_t** has) {
  const int64_t n = L.nrows;
  SX_CHECK(dev_alloc((void**)d, (size_t)std::max<int64_t>(n, 1) * sizeof(T)));
  int rc = dev_alloc((void**)has, (size_t)std::max<int64_t>(n, 1) * 4);
  if (rc != SX_OK) return rc;
  if (n > 0) {
    k_first_diag<T><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, n, *d,
                                                                 *has);
    ctx->launches++;
  }
  return SX_OK;
}

template <typename T>
int seq_sum(sx_ctx ctx, const T* a, const T* b, int64_t n, void* out_host) {
  T* dout = nullptr;
  SX_CHECK(dev_alloc((void**)&dout, 16));
  k_seq_sum<T><<<1, 32, 0, ctx->stream>>>(a, b, n, dout);
  ctx->launches++;
  cudaMemcpyAsync(out_host, dout, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream);
  const int rc = sync_check(ctx, "sequential sum");
  dev_free(dout);
  return rc;
}

template <typename T>
int trace_impl(sx_ctx ctx, sx_op a, void* out) {
  T* d = nullptr;
  int32_t* has = nullptr;
  int rc = first_diag<T>(ctx, a->sym_low->csr, &d, &has);
  if (rc == SX_OK) rc = seq_sum<T>(ctx, d, nullptr, a->nrows, out);
  dev_free(d);
  dev_free(has);
  return rc;
}

template <typename T>
int quad_impl(sx_ctx ctx, sx_op a, const void* x, sx_mem mem, void* out) {
  const int64_t n = a->nrows;
  T *dx = nullptr, *dy = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&dx, (size_t)std::max<int64_t>(n, 1) * sizeof(T)))) break;
    if ((rc = dev_alloc((void**)&dy, (size_t)std::max<int64_t>(n, 1) * sizeof(T)))) break;
    if (n > 0)
      SX_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(T),
                              mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              ctx->stream));
    if ((rc = launch_apply<T, EpiPlain<T>, true>(ctx, a, dx, dy, EpiPlain<T>{}))) break;
    rc = seq_sum<T>(ctx, dx, dy, n, out);
  } while (0);
  dev_free(dx);
  dev_free(dy);
  return rc;
}

template <typename T>
int rank1_impl(sx_ctx ctx, sx_op a, const void* x, sx_mem mem, double alpha) {
  const DevCsr& L = a->sym_low->csr;
  const int64_t n = L.nrows;
  const size_t nb = (size_t)std::max<int64_t>(n, 1);
  T* dx = nullptr;
  int32_t *cnt = nullptr, *np = nullptr, *ni = nullptr;
  T* nv = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&dx, nb * sizeof(T)))) break;
    if ((rc = dev_alloc((void**)&cnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&np, (nb + 1) * 4))) break;
    if (n > 0)
      SX_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(T),
                              mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              ctx->stream));
    const int g = (int)std::min<int64_t>(std::max<int64_t>(n, 1), (int64_t)ctx->num_sms * 8);
    if (n > 0) {
      k_rank1_count<T><<<g, 256, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, n, dx, (T)alpha, cnt);
      ctx->launches++;
    }
    if ((rc = exclusive_scan_i32(ctx, cnt, n, np))) break;
    int32_t nnz = 0;
    SX_CUDA(cudaMemcpyAsync(&nnz, np + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = sync_check(ctx, "rank-1 count"))) break;
    if ((rc = dev_alloc((void**)&ni, (size_t)std::max<int32_t>(nnz, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&nv, (size_t)std::max<int32_t>(nnz, 1) * sizeof(T)))) break;
    if (n > 0) {
      k_rank1_write<T><<<g, 256, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, n, dx, (T)alpha, np, ni,
                                                   nv);
      ctx->launches++;
    }
    if ((rc = sync_check(ctx, "rank-1 write"))) break;
    sx_op low = wrap_csr(ctx, a->dtype, n, nnz, np, ni, nv);
    np = nullptr;
    ni = nullptr;
    nv = nullptr;
    rc = replace_low(ctx, a, low);
  } while (0);
  dev_free(dx);
  dev_free(cnt);
  dev_free(np);
  dev_free(ni);
  dev_free(nv);
  return rc;
}

template <typename T>
int half_impl(sx_ctx ctx, sx_op a, const T* x, T* y) {
  const DevCsr& L = a->sym_low->csr;
  const int64_t n = L.nrows;
  if (n == 0) return SX_OK;
  SX_CUDA(cudaMemsetAsync(y, 0, n * sizeof(T), ctx->stream));
  k_sym_half<T><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const T*)L.vals, n, x, y);
  ctx->launches++;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

}  // namespace

int sym_half_spmv(sx_ctx ctx, sx_op a, const void* x, void* y) {
  if (a->dtype == SX_F64) return half_impl<double>(ctx, a, (const double*)x, (double*)y);
  return half_impl<float>(ctx, a, (const float*)x, (float*)y);
}

}  // namespace sx

using namespace sx;

extern "C" {

int sx_sym_csr_new(sx_ctx ctx, sx_dtype dtype, const void* data, uint64_t data_len, const uint64_t* indptr,
                   uint64_t indptr_len, const uint64_t* indices, uint64_t nnz, uint64_t nrows, uint64_t ncols,
                   sx_op* out) {
  if (!ctx || !out || (indptr_len > 0 && !indptr) || (nnz > 0 && !indices) || (data_len > 0 && !data))
    return err_arg("null argument");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  *out = nullptr;
  // checks in the order of SymCsrMatrix::new (sym_csr.rs:70-126)
  if (nrows != ncols) return err_value("Symmetric matrix must be square");
  if (indptr_len != nrows + 1)
    return err_value("indptr length (" + std::to_string(indptr_len) + ") must be equal to rows + 1 (" +
                     std::to_string(nrows + 1) + ")");
  if (data_len != nnz)
    return err_value("data length (" + std::to_string(data_len) + ") must match indices length (" +
                     std::to_string(nnz) + ")");
  if (indptr[nrows] != nnz)
    return err_value("Last indptr value (" + std::to_string(indptr[nrows]) + ") must equal nnz (" +
                     std::to_string(nnz) + ")");
  for (uint64_t i = 0; i < nrows; ++i) {
    const uint64_t s = indptr[i], e = indptr[i + 1];
    // the reference slices indices[s..e], which panics when s > e or e > nnz
    if (s > e || e > nnz)
      return set_error(SX_ERR_INCONSISTENT_DATA, "Inconsistent data: row pointers must be non-decreasing");
    for (uint64_t k = s; k < e; ++k) {
      const uint64_t c = indices[k];
      if (c >= ncols)
        return set_error(SX_ERR_INDEX_OUT_OF_BOUNDS,
                         "Index (" + std::to_string(i) + ", " + std::to_string(c) +
                             ") out of bounds for array with shape (" + std::to_string(nrows) + ", " +
                             std::to_string(ncols) + ")",
                         i, c, nrows, ncols);
      if (c > i) return err_value("Symmetric CSR should only store the lower triangular part");
    }
  }
  // the merged rows hold up to 2 nnz entries behind int32 row pointers
  if (2 * nnz > 2147483647ull || nrows > 2147483646ull)
    return set_error(SX_ERR_INDEX_CAST_OVERFLOW,
                     "Index value " + std::to_string(2 * nnz) + " cannot be represented in the target type i32",
                     2 * nnz);
  SX_CUDA(cudaSetDevice(ctx->device));
  const size_t w = elt_size(dtype);
  const int64_t n = (int64_t)nrows;
  std::vector<int32_t> ip(n + 1), ix((size_t)std::max<uint64_t>(nnz, 1));
  for (int64_t i = 0; i <= n; ++i) ip[i] = (int32_t)indptr[i];
  for (uint64_t k = 0; k < nnz; ++k) ix[k] = (int32_t)indices[k];
  int32_t *dp = nullptr, *di = nullptr;
  void* dv = nullptr;
  int rc = dev_alloc((void**)&dp, (size_t)(n + 1) * 4);
  if (rc == SX_OK) rc = dev_alloc((void**)&di, (size_t)std::max<uint64_t>(nnz, 1) * 4);
  if (rc == SX_OK) rc = dev_alloc(&dv, (size_t)std::max<uint64_t>(nnz, 1) * w);
  if (rc != SX_OK) {
    dev_free(dp);
    dev_free(di);
    dev_free(dv);
    return rc;
  }
  cudaMemcpyAsync(dp, ip.data(), (n + 1) * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (nnz > 0) {
    cudaMemcpyAsync(di, ix.data(), nnz * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dv, data, nnz * w, cudaMemcpyHostToDevice, ctx->stream);
  }
  sx_op low = wrap_csr(ctx, dtype, n, (int64_t)nnz, dp, di, dv);
  SX_CHECK(make_sym(ctx, low, out));
  return clear_error();
}

int sx_sym_csr_from_csr(sx_ctx ctx, sx_op a, sx_op* out) {
  if (!ctx || !a || !out) return err_arg("null argument");
  if (a->kind != SX_OP_CSR) return err_arg("not a CSR operator");
  *out = nullptr;
  // SymCsrMatrix::from_csr (sym_csr.rs:149-189)
  if (a->nrows != a->ncols) return err_value("Symmetric matrix must be square");
  SX_CUDA(cudaSetDevice(ctx->device));
  const DevCsr& A = a->csr;
  const int64_t n = A.nrows;
  const size_t nb = (size_t)std::max<int64_t>(n, 1);
  const int g = vec_grid(ctx, (int64_t)nb);
  int* bad = nullptr;
  int32_t *cnt = nullptr, *lp = nullptr, *li = nullptr;
  void* lv = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&bad, 16))) break;
    SX_CUDA(cudaMemsetAsync(bad, 0, 4, ctx->stream));
    if (n > 0) {
      // tolerance T::epsilon() * 100
      if (a->dtype == SX_F64)
        k_sym_check<double><<<g, kBlock, 0, ctx->stream>>>(A.indptr, A.indices, (const double*)A.vals, n,
                                                           2.220446049250313e-16 * 100.0, bad);
      else
        k_sym_check<float><<<g, kBlock, 0, ctx->stream>>>(A.indptr, A.indices, (const float*)A.vals, n,
                                                          1.1920928955078125e-07f * 100.0f, bad);
      ctx->launches++;
    }
    int hb = 0;
    SX_CUDA(cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = sync_check(ctx, "symmetry check"))) break;
    if (hb) {
      rc = err_value("Matrix must be symmetric to convert to SymCSR format");
      break;
    }
    if ((rc = dev_alloc((void**)&cnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&lp, (nb + 1) * 4))) break;
    if (n > 0) {
      k_lower_count<<<g, kBlock, 0, ctx->stream>>>(A.indptr, A.indices, n, cnt);
      ctx->launches++;
    }
    if ((rc = exclusive_scan_i32(ctx, cnt, n, lp))) break;
    int32_t lnnz = 0;
    SX_CUDA(cudaMemcpyAsync(&lnnz, lp + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = sync_check(ctx, "lower count"))) break;
    if ((rc = dev_alloc((void**)&li, (size_t)std::max<int32_t>(lnnz, 1) * 4))) break;
    if ((rc = dev_alloc(&lv, (size_t)std::max<int32_t>(lnnz, 1) * elt_size(a->dtype)))) break;
    if (n > 0) {
      if (a->dtype == SX_F64)
        k_lower_copy<double><<<g, kBlock, 0, ctx->stream>>>(A.indptr, A.indices, (const double*)A.vals, n, lp, li,
                                                            (double*)lv);
      else
        k_lower_copy<float><<<g, kBlock, 0, ctx->stream>>>(A.indptr, A.indices, (const float*)A.vals, n, lp, li,
                                                           (float*)lv);
      ctx->launches++;
    }
    if ((rc = sync_check(ctx, "lower copy"))) break;
    sx_op low = wrap_csr(ctx, a->dtype, n, lnnz, lp, li, lv);
    lp = nullptr;
    li = nullptr;
    lv = nullptr;
    rc = make_sym(ctx, low, out);
  } while (0);
  dev_free(bad);
  dev_free(cnt);
  dev_free(lp);
  dev_free(li);
  dev_free(lv);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_sym_csr_info(sx_ctx ctx, sx_op a, uint64_t* nnz_stored, uint64_t* nnz_full) {
  if (!ctx || !is_sym(a)) return err_arg("not a symmetric CSR operator");
  const DevCsr& L = a->sym_low->csr;
  if (nnz_stored) *nnz_stored = (uint64_t)L.nnz;  // SymCsrMatrix::nnz_stored = data.len()
  if (nnz_full) {
    // SymCsrMatrix::nnz (sym_csr.rs:254-268): rows that store a diagonal
    // entry count once, every other stored entry twice
    SX_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = L.nrows;
    void* d = nullptr;
    int32_t* has = nullptr;
    int rc = a->dtype == SX_F64 ? first_diag<double>(ctx, L, (double**)&d, &has)
                                : first_diag<float>(ctx, L, (float**)&d, &has);
    std::vector<int32_t> h((size_t)std::max<int64_t>(n, 1));
    if (rc == SX_OK && n > 0) {
      cudaMemcpyAsync(h.data(), has, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
      rc = sync_check(ctx, "diagonal count");
    }
    dev_free(d);
    dev_free(has);
    SX_CHECK(rc);
    uint64_t diag = 0;
    for (int64_t i = 0; i < n; ++i) diag += (uint64_t)h[i];
    *nnz_full = diag + 2 * ((uint64_t)L.nnz - diag);
  }
  return clear_error();
}

int sx_sym_csr_download(sx_ctx ctx, sx_op a, uint64_t* indptr, uint64_t* indices, void* data) {
  if (!ctx || !is_sym(a)) return err_arg("not a symmetric CSR operator");
  // the public data / indptr / indices fields (sym_csr.rs:28-34)
  return sx_csr_download(ctx, a->sym_low, indptr, indices, data);
}

int sx_sym_csr_to_csr(sx_ctx ctx, sx_op a, sx_op* out) {
  if (!ctx || !out || !is_sym(a)) return err_arg("not a symmetric CSR operator");
  SX_CUDA(cudaSetDevice(ctx->device));
  // SymCsrMatrix::to_csr (sym_csr.rs:305-337): triplets (i, j, v) and, off
  // the diagonal, (j, i, v) in stored order, then CsrMatrix::new
  const DevCsr& L = a->sym_low->csr;
  const int64_t n = L.nrows;
  const size_t w = elt_size(a->dtype);
  std::vector<int32_t> ip(n + 1), ix((size_t)std::max<int64_t>(L.nnz, 1));
  std::vector<char> v((size_t)std::max<int64_t>(L.nnz, 1) * w);
  SX_CUDA(cudaMemcpyAsync(ip.data(), L.indptr, (n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (L.nnz > 0) {
    SX_CUDA(cudaMemcpyAsync(ix.data(), L.indices, L.nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(v.data(), L.vals, L.nnz * w, cudaMemcpyDeviceToHost, ctx->stream));
  }
  SX_CHECK(sync_check(ctx, "to_csr download"));
  std::vector<uint64_t> rows, cols;
  std::vector<char> data;
  rows.reserve(2 * L.nnz);
  cols.reserve(2 * L.nnz);
  data.reserve(2 * L.nnz * w);
  for (int64_t i = 0; i < n; ++i)
    for (int32_t k = ip[i]; k < ip[i + 1]; ++k) {
      rows.push_back((uint64_t)i);
      cols.push_back((uint64_t)ix[k]);
      data.insert(data.end(), v.begin() + (size_t)k * w, v.begin() + (size_t)(k + 1) * w);
      if (ix[k] != i) {
        rows.push_back((uint64_t)ix[k]);
        cols.push_back((uint64_t)i);
        data.insert(data.end(), v.begin() + (size_t)k * w, v.begin() + (size_t)(k + 1) * w);
      }
    }
  return sx_csr_from_triplets(ctx, (sx_dtype)a->dtype, SX_API_CSR_MATRIX, rows.data(), cols.data(), data.data(),
                              rows.size(), (uint64_t)n, (uint64_t)n, 0, out);
}

int sx_sym_csr_trace(sx_ctx ctx, sx_op a, void* out_value) {
  if (!ctx || !out_value || !is_sym(a)) return err_arg("not a symmetric CSR operator");
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(a->dtype == SX_F64 ? trace_impl<double>(ctx, a, out_value) : trace_impl<float>(ctx, a, out_value));
  return clear_error();
}

int sx_sym_csr_quadratic_form(sx_ctx ctx, sx_op a, const void* x, uint64_t x_len, sx_mem mem, void* out_value) {
  if (!ctx || !out_value || !is_sym(a) || (x_len > 0 && !x)) return err_arg("not a symmetric CSR operator");
  if (x_len != (uint64_t)a->nrows) return err_dim((uint64_t)a->nrows, x_len);
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(a->dtype == SX_F64 ? quad_impl<double>(ctx, a, x, mem, out_value)
                              : quad_impl<float>(ctx, a, x, mem, out_value));
  return clear_error();
}

int sx_sym_csr_rank1_update(sx_ctx ctx, sx_op a, const void* x, uint64_t x_len, double alpha, sx_mem mem) {
  if (!ctx || !is_sym(a) || (x_len > 0 && !x)) return err_arg("not a symmetric CSR operator");
  if (x_len != (uint64_t)a->nrows) return err_dim((uint64_t)a->nrows, x_len);
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(a->dtype == SX_F64 ? rank1_impl<double>(ctx, a, x, mem, alpha) : rank1_impl<float>(ctx, a, x, mem, alpha));
  return clear_error();
}

}  // extern "C"
