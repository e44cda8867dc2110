// IC(0) preconditioner on the device (scirs2-sparse/src/linalg/ic.rs:15-230).
//
// Factorisation and triangular solves are dependency-driven: rows are handed
// to warps in order through an atomic counter, and a row waits only on rows
// handed out before it (already running), so progress is guaranteed.  Each
// wait polls a ready flag and gives up after kWaitNs nanoseconds by raising an
// abort flag that ends every other wait at once; the host turns it into
// SX_ERR_DEVICE_TIMEOUT.  No input can keep a kernel spinning indefinitely.
//
// Exactness: the reference factorisation runs its loops in lane 0 of the
// row's warp in the reference's order (bit-identical).  The solves gather the
// products of a row in parallel and lane 0 subtracts them in storage order:
//   forward  z_i = (x_i - sum_{j<i} L_ij z_j) / L_ii(last diagonal entry)
//   backward y_i = (z_i - sum_{j>i, ascending} L_ji y_j) / L_ii(first)
// where L_ji is the first entry of row j with column i (ic.rs:154-217); the
// backward solve walks a transposed copy of those first entries.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"
#include "sx_sync.cuh"

namespace sx {

struct IC0Dev {
  DevCsr L;              // lower part of A in storage order, factorised in place
  sx_op lt = nullptr;    // first strictly-lower entries, transposed (backward solve)
  void* dlast = nullptr; // forward-solve diagonal: last diagonal entry of each row
  void* dfirst = nullptr;// backward-solve diagonal: first diagonal entry
  void* z = nullptr;     // forward-solve result
  int* ready = nullptr;  // 2 * n flags (forward, backward)
  int* ctl = nullptr;    // [0] row counter fwd, [1] row counter bwd, [2] abort, [3] spare
  // rows in dependency-level order (forward: levels of L; backward: of L^T);
  // the counters hand rows out in this order
  int32_t* fwd_order = nullptr;
  int32_t* bwd_order = nullptr;
  int variant = 0;
};

void ic0_destroy(IC0Dev* p) {
  if (!p) return;
  dev_free(p->L.indptr);
  dev_free(p->L.indices);
  dev_free(p->L.vals);
  dev_free(p->L.tile_row);
  free_sliced(p->L);
  dev_free(p->L.col16);
  dev_free(p->L.chunk_base);
  dev_free(p->L.vals16);
  if (p->lt) destroy_op_internal(p->lt);
  dev_free(p->dlast);
  dev_free(p->dfirst);
  dev_free(p->z);
  dev_free(p->ready);
  dev_free(p->ctl);
  dev_free(p->fwd_order);
  dev_free(p->bwd_order);
  delete p;
}

namespace {

// per-row error record: err[0] = smallest failing row (or INT_MAX), err_code[row]
enum : int { E_NONE = 0, E_MISSING_DIAG = 1, E_NOT_PD = 2 };

// ---- reference factorisation (ic.rs:52-129), lane 0 of a warp per row
template <typename T>
__global__ void k_ic0_factor_ref(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                                 T* ld, int64_t n, int* ready, int* ctl, int* err_row,
                                 int* err_code, const int32_t* __restrict__ order, unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int64_t i = 0;
    if (lane == 0) i = atomicAdd(ctl + 0, 1);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= n) return;
    i = order[i];
    if (lane == 0) {
      const int32_t rs = lp[i], re = lp[i + 1];
      int32_t di = -1;
      for (int32_t k = rs; k < re; ++k)
        if (li[k] == (int32_t)i) { di = k; break; }
      if (di < 0) {
        err_code[i] = E_MISSING_DIAG;
        atomicMin(err_row, (int)i);
      } else {
        T dv = ldv(ld + di);
        for (int32_t k = rs; k < di; ++k) {
          const int32_t j = li[k];
          if (!wait_flag(ready + j, ctl + 2, wait_ns)) break;
          T ljj = T(0);
          for (int32_t q = lp[j]; q < lp[j + 1]; ++q)
            if (li[q] == j) { ljj = ldv(ld + q); break; }
          const T lk = ldv(ld + k);
          dv = sub_rn(dv, mul_rn(lk, lk) / ljj);
        }
        if (dv <= T(0)) {
          err_code[i] = E_NOT_PD;
          atomicMin(err_row, (int)i);
        }
        const T dsq = sqrt(dv);
        ld[di] = dsq;
        // entries stored after the diagonal (only with unsorted or
        // duplicated input): ic.rs:107-128
        for (int32_t k = di + 1; k < re; ++k) {
          const int32_t j = li[k];
          if (j < (int32_t)i && !wait_flag(ready + j, ctl + 2, wait_ns)) break;
          T sum = T(0);
          for (int32_t p = rs; p < di; ++p) {
            const int32_t cp = li[p];
            for (int32_t q = lp[j]; q < lp[j + 1]; ++q)
              if (li[q] == cp) { sum = add_rn(sum, mul_rn(ldv(ld + p), ldv(ld + q))); break; }
          }
          ld[k] = (ldv(ld + k) - sum) / dsq;
        }
      }
      publish(ready + i);
    }
    __syncwarp();
  }
}

// ---- textbook IC(0) on sorted rows without duplicates:
// L_ij = (a_ij - sum_{m<j} L_im L_jm) / L_jj,  L_ii = sqrt(a_ii - sum_{m<i} L_im^2)
template <typename T>
__global__ void k_ic0_factor_textbook(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                                      T* ld, int64_t n, int* ready, int* ctl, int* err_row,
                                      int* err_code, const int32_t* __restrict__ order,
                                      unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int64_t i = 0;
    if (lane == 0) i = atomicAdd(ctl + 0, 1);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= n) return;
    i = order[i];
    if (lane == 0) {
      const int32_t rs = lp[i], re = lp[i + 1];
      const int32_t di = re - 1;
      if (re == rs || li[di] != (int32_t)i) {
        err_code[i] = E_MISSING_DIAG;
        atomicMin(err_row, (int)i);
      } else {
        T dsum = T(0);
        for (int32_t k = rs; k < di; ++k) {
          const int32_t j = li[k];
          if (!wait_flag(ready + j, ctl + 2, wait_ns)) break;
          T s = ldv(ld + k);
          int32_t p = rs, q = lp[j];
          const int32_t qe = lp[j + 1] - 1;  // row j without its diagonal
          while (p < k && q < qe) {
            const int32_t cp = li[p], cq = li[q];
            if (cp == cq) { s -= ldv(ld + p) * ldv(ld + q); ++p; ++q; }
            else if (cp < cq) ++p;
            else ++q;
          }
          const T l = s / ldv(ld + qe);
          ld[k] = l;
          dsum += l * l;
        }
        const T dv = ldv(ld + di) - dsum;
        if (!(dv > T(0))) {
          err_code[i] = E_NOT_PD;
          atomicMin(err_row, (int)i);
        }
        ld[di] = sqrt(dv);
      }
      publish(ready + i);
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void k_diag_first_last(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                                  const T* __restrict__ ld, int64_t n, T* dfirst, T* dlast) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    T f = T(1), l = T(1);
    bool seen = false;
    for (int32_t k = lp[r]; k < lp[r + 1]; ++k)
      if (li[k] == (int32_t)r) {
        if (!seen) { f = ld[k]; seen = true; }
        l = ld[k];
      }
    dfirst[r] = f;
    dlast[r] = l;
  }
}

// first strictly-lower occurrence of each column within a row
__global__ void k_first_strict_count(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                                     int64_t n, int32_t* cnt) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t c = 0;
    for (int32_t k = lp[r]; k < lp[r + 1]; ++k) {
      if (li[k] >= (int32_t)r) continue;
      bool dup = false;
      for (int32_t q = lp[r]; q < k; ++q)
        if (li[q] == li[k]) { dup = true; break; }
      c += !dup;
    }
    cnt[r] = c;
  }
}

template <typename T>
__global__ void k_first_strict_copy(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                                    const T* __restrict__ ld, int64_t n,
                                    const int32_t* __restrict__ sp, int32_t* si, T* sv) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t o = sp[r];
    for (int32_t k = lp[r]; k < lp[r + 1]; ++k) {
      if (li[k] >= (int32_t)r) continue;
      bool dup = false;
      for (int32_t q = lp[r]; q < k; ++q)
        if (li[q] == li[k]) { dup = true; break; }
      if (!dup) { si[o] = li[k]; sv[o] = ld[k]; ++o; }
    }
  }
}

// ---- forward solve L z = x (ic.rs:154-174), warp per row, in order
template <typename T>
__global__ void k_ic0_forward(const int32_t* __restrict__ lp, const int32_t* __restrict__ li,
                              const T* __restrict__ ld, const T* __restrict__ dlast, int64_t n,
                              const T* __restrict__ x, T* z, int* ready, int* ctl,
                              const int32_t* __restrict__ order, unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int64_t i = 0;
    if (lane == 0) i = atomicAdd(ctl + 0, 1);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= n) return;
    i = order[i];
    const int32_t rs = lp[i], re = lp[i + 1];
    T sum = x[i];
    for (int32_t base = rs; base < re; base += 32) {
      const int32_t k = base + lane;
      T prod = T(0);
      bool sub = false;
      if (k < re) {
        const int32_t j = li[k];
        if (j < (int32_t)i) {
          wait_flag(ready + j, ctl + 2, wait_ns);
          prod = mul_rn(ld[k], ldv(z + j));
          sub = true;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, sub);
      // lane 0 subtracts the products in storage order
      for (int t = 0; t < 32; ++t) {
        const T pt = __shfl_sync(0xffffffffu, prod, t);
        if (lane == 0 && ((m >> t) & 1u)) sum = sub_rn(sum, pt);
      }
    }
    if (lane == 0) {
      z[i] = sum / dlast[i];
      publish(ready + i);
    }
    __syncwarp();
  }
}

// ---- backward solve L^T y = z (ic.rs:177-217) over the transposed first
// entries, rows handed out from the last one down
template <typename T>
__global__ void k_ic0_backward(const int32_t* __restrict__ tp, const int32_t* __restrict__ ti,
                               const T* __restrict__ tv, const T* __restrict__ dfirst, int64_t n,
                               const T* __restrict__ z, T* y, int* ready, int* ctl,
                               const int32_t* __restrict__ order, unsigned long long wait_ns) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int64_t q = 0;
    if (lane == 0) q = atomicAdd(ctl + 1, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= n) return;
    const int64_t i = order[q];
    const int32_t rs = tp[i], re = tp[i + 1];
    T sum = ldv(z + i);
    for (int32_t base = rs; base < re; base += 32) {
      const int32_t k = base + lane;
      T prod = T(0);
      const bool act = k < re;
      if (act) {
        const int32_t j = ti[k];  // j > i
        wait_flag(ready + j, ctl + 2, wait_ns);
        prod = mul_rn(tv[k], ldv(y + j));
      }
      const unsigned m = __ballot_sync(0xffffffffu, act);
      for (int t = 0; t < 32; ++t) {
        const T pt = __shfl_sync(0xffffffffu, prod, t);
        if (lane == 0 && ((m >> t) & 1u)) sum = sub_rn(sum, pt);
      }
    }
    if (lane == 0) {
      y[i] = sum / dfirst[i];
      publish(ready + i);
    }
    __syncwarp();
  }
}

int solve_grid(sx_ctx ctx) { return ctx->num_sms * 8; }

}  // namespace

int ic0_apply(sx_ctx ctx, sx_op op, const void* x, void* y) {
  IC0Dev* d = op->ic0;
  const int64_t n = op->nrows;
  if (n <= 0) return SX_OK;
  SX_CUDA(cudaMemsetAsync(d->ready, 0, 2 * n * sizeof(int), ctx->stream));
  SX_CUDA(cudaMemsetAsync(d->ctl, 0, 2 * sizeof(int), ctx->stream));
  const DevCsr& L = d->L;
  const DevCsr& T = d->lt->csr;
  const int g = solve_grid(ctx);
  if (op->dtype == SX_F64) {
    k_ic0_forward<double><<<g, kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const double*)L.vals,
                                                         (const double*)d->dlast, n, (const double*)x,
                                                         (double*)d->z, d->ready, d->ctl, d->fwd_order, ctx->wait_ns);
    k_ic0_backward<double><<<g, kBlock, 0, ctx->stream>>>(T.indptr, T.indices, (const double*)T.vals,
                                                          (const double*)d->dfirst, n,
                                                          (const double*)d->z, (double*)y,
                                                          d->ready + n, d->ctl, d->bwd_order, ctx->wait_ns);
  } else {
    k_ic0_forward<float><<<g, kBlock, 0, ctx->stream>>>(L.indptr, L.indices, (const float*)L.vals,
                                                        (const float*)d->dlast, n, (const float*)x,
                                                        (float*)d->z, d->ready, d->ctl, d->fwd_order, ctx->wait_ns);
    k_ic0_backward<float><<<g, kBlock, 0, ctx->stream>>>(T.indptr, T.indices, (const float*)T.vals,
                                                         (const float*)d->dfirst, n,
                                                         (const float*)d->z, (float*)y,
                                                         d->ready + n, d->ctl, d->bwd_order, ctx->wait_ns);
  }
  ctx->launches += 2;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

// a wait on a flag that nothing sets: ends only by its limit
__global__ void k_wait_selftest(int* flags, unsigned long long wait_ns, unsigned long long* waited) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned long long t0 = globaltimer();
  const bool ok = wait_flag(flags + 0, flags + 1, wait_ns);
  waited[0] = globaltimer() - t0;
  flags[2] = ok ? 1 : 0;
}

int ctx_set_wait_limit(sx_ctx ctx, uint64_t ns) {
  ctx->wait_ns = ns ? (unsigned long long)ns : 2000000000ull;
  return SX_OK;
}

int wait_selftest(sx_ctx ctx, uint64_t* waited_ns) {
  int* flags = nullptr;
  SX_CHECK(dev_alloc((void**)&flags, 4 * sizeof(int) + 8));
  unsigned long long* waited = (unsigned long long*)(flags + 4);
  int rc = SX_OK;
  do {
    if (cudaMemsetAsync(flags, 0, 4 * sizeof(int) + 8, ctx->stream) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "selftest memset", __FILE__, __LINE__);
      break;
    }
    k_wait_selftest<<<1, 32, 0, ctx->stream>>>(flags, ctx->wait_ns, waited);
    ctx->launches++;
    int h[3] = {0, 0, 0};
    unsigned long long w = 0;
    cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&w, waited, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "wait selftest", __FILE__, __LINE__);
      break;
    }
    if (waited_ns) *waited_ns = w;
    if (!h[2]) rc = set_error(SX_ERR_DEVICE_TIMEOUT, "Device timeout: the self-test wait gave up at its limit");
  } while (0);
  dev_free(flags);
  return rc;
}

// abort flag of an IC(0) operator: a wait that gave up
// (also of the ILU(0) and SSOR sweeps, which use the same waits)
int ic0_health(sx_ctx ctx, sx_op op) {
  if (!op) return SX_OK;
  const int* ctl = nullptr;
  if (op->kind == SX_OP_IC0 && op->ic0) ctl = op->ic0->ctl;
  else if (op->kind == SX_OP_ILU0 || op->kind == SX_OP_SSOR) ctl = tri_ctl(op);
  if (!ctl) return SX_OK;
  int h[4] = {0, 0, 0, 0};
  SX_CUDA(cudaMemcpyAsync(h, ctl, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  // read and clear: the next call on this operator starts without the abort
  if (h[2]) SX_CUDA(cudaMemsetAsync((void*)(ctl + 2), 0, sizeof(int), ctx->stream));
  if (h[2])
    return set_error(SX_ERR_DEVICE_TIMEOUT,
                     op->kind == SX_OP_IC0
                         ? "Device timeout: an IC(0) dependency wait exceeded its time limit"
                         : "Device timeout: a triangular-sweep dependency wait exceeded its time limit");
  return SX_OK;
}


// Rows sorted by dependency level (a stable counting sort): forward, a row
// depends on the rows j < i of its pattern; backward, on the rows j > i.  A
// row's dependencies sit on lower levels, so they are handed out before it.
int level_order(sx_ctx ctx, const DevCsr& c, bool forward, int32_t** out) {
  const int64_t n = c.nrows;
  std::vector<int32_t> ptr(n + 1), idx(std::max<int64_t>(c.nnz, 1));
  SX_CUDA(cudaMemcpyAsync(ptr.data(), c.indptr, (n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (c.nnz > 0)
    SX_CUDA(cudaMemcpyAsync(idx.data(), c.indices, c.nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> lev(n, 0);
  int32_t maxl = 0;
  for (int64_t t = 0; t < n; ++t) {
    const int64_t i = forward ? t : n - 1 - t;
    int32_t l = 0;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int32_t j = idx[k];
      if (forward ? (j < i) : (j > i)) l = std::max(l, lev[j] + 1);
    }
    lev[i] = l;
    maxl = std::max(maxl, l);
  }
  std::vector<int64_t> start(maxl + 2, 0);
  for (int64_t i = 0; i < n; ++i) start[lev[i] + 1]++;
  for (int32_t l = 0; l <= maxl; ++l) start[l + 1] += start[l];
  std::vector<int32_t> order(std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n; ++i) order[start[lev[i]]++] = (int32_t)i;
  SX_CHECK(dev_alloc((void**)out, std::max<int64_t>(n, 1) * 4));
  SX_CUDA(cudaMemcpyAsync(*out, order.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return SX_OK;
}

}  // namespace sx

using namespace sx;

extern "C" int sx_ctx_set_wait_limit(sx_ctx ctx, uint64_t ns) {
  if (!ctx) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx");
  return ctx_set_wait_limit(ctx, ns) == SX_OK ? clear_error() : SX_ERR_INVALID_ARGUMENT;
}

extern "C" int sx_wait_selftest(sx_ctx ctx, uint64_t* waited_ns) {
  if (!ctx) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int rc = wait_selftest(ctx, waited_ns);
  return rc == SX_OK ? clear_error() : rc;
}

extern "C" int sx_precond_ic0(sx_ctx ctx, sx_op a, int variant, sx_op* out) {
  if (!ctx || !a || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a->kind != SX_OP_CSR) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: not CSR");
  if (variant != SX_IC0_REFERENCE && variant != SX_IC0_TEXTBOOK)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: IC0 variant");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a->nrows;
  if (n != a->ncols)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(n) + ", found " +
                         std::to_string(a->ncols),
                     (uint64_t)n, (uint64_t)a->ncols);
  if (!a->csr.monotone)
    return set_error(SX_ERR_INCONSISTENT_DATA,
                     "Inconsistent data: IC0 needs non-decreasing row pointers");
  if (variant == SX_IC0_TEXTBOOK && !a->csr.has_sorted_indices)
    return set_error(SX_ERR_VALUE, "Value error: textbook IC(0) needs sorted column indices");
  const size_t w = elt_size(a->dtype);
  IC0Dev* d = new IC0Dev();
  d->variant = variant;
  int32_t *cnt = nullptr, *scnt = nullptr, *sp = nullptr, *si = nullptr;
  void* sv = nullptr;
  int *err = nullptr, *codes = nullptr;
  int rc = SX_OK;
  const int g = vec_grid(ctx, n);
  do {
    const size_t nb = std::max<int64_t>(n, 1);
    if ((rc = dev_alloc((void**)&cnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&d->L.indptr, (nb + 1) * 4))) break;
    if (n > 0) {
      k_lower_count<<<g, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, n, cnt);
      ctx->launches++;
    }
    if ((rc = exclusive_scan_i32(ctx, cnt, n, d->L.indptr))) break;
    int32_t lnnz = 0;
    SX_CUDA(cudaMemcpy(&lnnz, d->L.indptr + n, 4, cudaMemcpyDeviceToHost));
    d->L.nrows = d->L.ncols = n;
    d->L.nnz = lnnz;
    if ((rc = dev_alloc((void**)&d->L.indices, std::max<int32_t>(lnnz, 1) * 4))) break;
    if ((rc = dev_alloc(&d->L.vals, std::max<int32_t>(lnnz, 1) * w))) break;
    if (n > 0) {
      if (a->dtype == SX_F64)
        k_lower_copy<double><<<g, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices,
                                                            (const double*)a->csr.vals, n,
                                                            d->L.indptr, d->L.indices, (double*)d->L.vals);
      else
        k_lower_copy<float><<<g, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices,
                                                           (const float*)a->csr.vals, n,
                                                           d->L.indptr, d->L.indices, (float*)d->L.vals);
      ctx->launches++;
    }
    if ((rc = level_order(ctx, d->L, true, &d->fwd_order))) break;
    if ((rc = dev_alloc((void**)&d->ready, 2 * nb * sizeof(int)))) break;
    if ((rc = dev_alloc((void**)&d->ctl, 4 * sizeof(int)))) break;
    if ((rc = dev_alloc((void**)&err, sizeof(int)))) break;
    if ((rc = dev_alloc((void**)&codes, nb * sizeof(int)))) break;
    SX_CUDA(cudaMemsetAsync(d->ready, 0, 2 * nb * sizeof(int), ctx->stream));
    SX_CUDA(cudaMemsetAsync(d->ctl, 0, 4 * sizeof(int), ctx->stream));
    SX_CUDA(cudaMemsetAsync(codes, 0, nb * sizeof(int), ctx->stream));
    int big = 0x7fffffff;
    SX_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (n > 0) {
      const int sg = solve_grid(ctx);
      if (a->dtype == SX_F64) {
        if (variant == SX_IC0_REFERENCE)
          k_ic0_factor_ref<double><<<sg, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (double*)d->L.vals, n, d->ready, d->ctl, err, codes, d->fwd_order, ctx->wait_ns);
        else
          k_ic0_factor_textbook<double><<<sg, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (double*)d->L.vals, n, d->ready, d->ctl, err, codes, d->fwd_order, ctx->wait_ns);
      } else {
        if (variant == SX_IC0_REFERENCE)
          k_ic0_factor_ref<float><<<sg, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (float*)d->L.vals, n, d->ready, d->ctl, err, codes, d->fwd_order, ctx->wait_ns);
        else
          k_ic0_factor_textbook<float><<<sg, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (float*)d->L.vals, n, d->ready, d->ctl, err, codes, d->fwd_order, ctx->wait_ns);
      }
      ctx->launches++;
    }
    int herr = 0, hctl[4] = {0, 0, 0, 0};
    SX_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(hctl, d->ctl, sizeof(hctl), cudaMemcpyDeviceToHost, ctx->stream));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "IC0 factorisation", __FILE__, __LINE__); break; }
    if (hctl[2]) {
      rc = set_error(SX_ERR_DEVICE_TIMEOUT, "Device timeout: IC(0) factorisation wait exceeded its limit");
      break;
    }
    if (herr != 0x7fffffff) {
      int code = 0;
      SX_CUDA(cudaMemcpy(&code, codes + herr, sizeof(int), cudaMemcpyDeviceToHost));
      if (code == E_MISSING_DIAG)
        rc = set_error(SX_ERR_VALUE, "Value error: Missing diagonal element at position " + std::to_string(herr));
      else
        rc = set_error(SX_ERR_VALUE, "Value error: Matrix is not positive definite or factorization broke down");
      break;
    }
    if ((rc = dev_alloc(&d->dfirst, nb * w))) break;
    if ((rc = dev_alloc(&d->dlast, nb * w))) break;
    if ((rc = dev_alloc(&d->z, nb * w))) break;
    if ((rc = dev_alloc((void**)&scnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&sp, (nb + 1) * 4))) break;
    if (a->dtype == SX_F64)
      k_diag_first_last<double><<<g, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (const double*)d->L.vals, n, (double*)d->dfirst, (double*)d->dlast);
    else
      k_diag_first_last<float><<<g, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (const float*)d->L.vals, n, (float*)d->dfirst, (float*)d->dlast);
    k_first_strict_count<<<g, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, n, scnt);
    ctx->launches += 2;
    if ((rc = exclusive_scan_i32(ctx, scnt, n, sp))) break;
    int32_t snnz = 0;
    SX_CUDA(cudaMemcpy(&snnz, sp + n, 4, cudaMemcpyDeviceToHost));
    if ((rc = dev_alloc((void**)&si, std::max<int32_t>(snnz, 1) * 4))) break;
    if ((rc = dev_alloc(&sv, std::max<int32_t>(snnz, 1) * w))) break;
    if (a->dtype == SX_F64)
      k_first_strict_copy<double><<<g, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (const double*)d->L.vals, n, sp, si, (double*)sv);
    else
      k_first_strict_copy<float><<<g, kBlock, 0, ctx->stream>>>(d->L.indptr, d->L.indices, (const float*)d->L.vals, n, sp, si, (float*)sv);
    ctx->launches++;
    // transpose of the strictly-lower first entries: rows of L^T, ascending j
    sx_op s = new sx_op_s();
    s->kind = SX_OP_CSR;
    s->dtype = a->dtype;
    s->device = ctx->device;
    s->nrows = s->ncols = n;
    s->csr.nrows = s->csr.ncols = n;
    s->csr.nnz = snnz;
    s->csr.indptr = sp;
    s->csr.indices = si;
    s->csr.vals = sv;
    sp = nullptr; si = nullptr; sv = nullptr;
    rc = csr_transpose_internal(ctx, s, &d->lt);
    destroy_op_internal(s);
    if (rc) break;
    if ((rc = level_order(ctx, d->lt->csr, false, &d->bwd_order))) break;
    rc = csr_finalize_stats(ctx, d->L);
  } while (0);
  dev_free(cnt); dev_free(scnt); dev_free(sp); dev_free(si); dev_free(sv);
  dev_free(err); dev_free(codes);
  if (rc != SX_OK) {
    ic0_destroy(d);
    return rc;
  }
  sx_op op = new sx_op_s();
  op->kind = SX_OP_IC0;
  op->dtype = a->dtype;
  op->device = ctx->device;
  op->nrows = op->ncols = n;
  op->ic0 = d;
  op->serial = next_op_serial();
  *out = op;
  return clear_error();
}
