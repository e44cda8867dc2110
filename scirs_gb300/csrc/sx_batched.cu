// Batched preconditioned CG over thousands of independent SPD systems of
// uneven size (no reference counterpart: the reference solves one system per
// cg call, linalg/iterative.rs:40-162, and this batches that loop).
//
// Layout: the systems form one block-diagonal CSR (global row and column
// numbering); system s owns rows [sys_ptr[s], sys_ptr[s+1]).  Work items are
// blocks of up to 256 consecutive rows of one system.  Each CG phase is one
// persistent kernel that walks the list of blocks whose system is still
// running; per-system reductions end in the last block of that system to
// finish (a per-system ticket), which sums the system's block partials in a
// fixed order and performs the reference cg's scalar step for that system.
// After each iteration a compaction kernel drops the blocks of finished
// systems and re-arms the CUDA-graph WHILE condition.
//
// Mixed precision: an outer FP64 loop forms r = b - A x per system in FP64,
// retires systems whose true relative residual meets the tolerance, and runs
// the batched FP32 Jacobi-PCG on the rest for the correction.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"

namespace sx {
namespace {

constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;

struct BatchPlan {
  int64_t nsys = 0, nblocks = 0, nrows = 0;
  int32_t* blk_sys = nullptr;
  int32_t* blk_row0 = nullptr;
  int32_t* blk_nrows = nullptr;
  int32_t* sys_fb = nullptr;   // first block of each system
  int32_t* sys_nb = nullptr;   // blocks of each system
  int32_t* lists = nullptr;    // 2 x nblocks active-block lists
  int32_t* ctl = nullptr;      // [0] cur list, [1] count list0, [2] count list1, [3] running,
                               // [4] budget, [5] use_cond, [6] ticket, [7] pad
  unsigned int* sys_ticket = nullptr;  // per-system last-block counters
  void* partials = nullptr;    // 3 * nblocks values
  unsigned long long* cond = nullptr;  // conditional handle
};

template <typename T>
struct SysState {
  T *rz_old, *alpha, *beta, *rnorm, *tol;
  int *status, *message, *converged;
  unsigned long long* iterations;
  unsigned long long max_iter;
};

struct PlanView {
  const int32_t *blk_sys, *blk_row0, *blk_nrows, *sys_fb, *sys_nb;
  int32_t* lists;
  int32_t* ctl;
  unsigned int* ticket;
  int64_t nblocks;
  const unsigned long long* cond;
};

// Block-wide sum of three values (valid in all threads).
template <typename T>
__device__ Acc3<T> bsum3(Acc3<T> v) { return block_sum3<T>(v); }

// Per-system reduction tail: write this block's partials, take the system's
// ticket; the last block sums the system's partials in block order.
template <typename T>
__device__ bool sys_reduce(const PlanView& pv, T* partials, int b, int s, Acc3<T> v, Acc3<T>& tot) {
  __shared__ bool s_last;
  Acc3<T> bs = bsum3(v);
  if (threadIdx.x == 0) {
    partials[3 * b + 0] = bs.a;
    partials[3 * b + 1] = bs.b;
    partials[3 * b + 2] = bs.c;
    __threadfence();
    unsigned t = atomicAdd(pv.ticket + s, 1u);
    s_last = (t == (unsigned)pv.sys_nb[s] - 1u);
  }
  __syncthreads();
  const bool last = s_last;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  Acc3<T> acc{T(0), T(0), T(0)};
  const int fb = pv.sys_fb[s], nb = pv.sys_nb[s];
  for (int j = threadIdx.x; j < nb; j += kBlock) {
    acc.a += __ldcg(partials + 3 * (fb + j) + 0);
    acc.b += __ldcg(partials + 3 * (fb + j) + 1);
    acc.c += __ldcg(partials + 3 * (fb + j) + 2);
  }
  tot = bsum3(acc);
  if (threadIdx.x == 0) pv.ticket[s] = 0u;
  return true;
}

// -------------------------------------------------------- CG phase kernels
// A p for a block's rows (exact per-row order) with p.Ap; finalize alpha.
template <typename T>
__global__ void __launch_bounds__(kBlock) kb_spmv_pap(PlanView pv, const int32_t* __restrict__ indptr,
                                                       const int32_t* __restrict__ indices,
                                                       const T* __restrict__ vals, const T* __restrict__ p,
                                                       T* q, T* partials, SysState<T> st) {
  __shared__ int32_t s_ptr[kBlock + 1];
  __shared__ T s_prod[kTile];
  const int cur = pv.ctl[0];
  const int cnt = pv.ctl[1 + cur];
  const int32_t* list = pv.lists + (int64_t)cur * pv.nblocks;
  const int tid = threadIdx.x;
  for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
    const int b = list[w];
    const int s = pv.blk_sys[b];
    const int64_t r0 = pv.blk_row0[b];
    const int nr = pv.blk_nrows[b];
    if (tid <= nr) s_ptr[tid] = indptr[r0 + tid];
    if (tid == 0 && nr == kBlock) s_ptr[kBlock] = indptr[r0 + kBlock];
    __syncthreads();
    const int32_t s0 = s_ptr[0], e0 = s_ptr[nr];
    int32_t my_s = 0, my_e = 0;
    if (tid < nr) { my_s = s_ptr[tid]; my_e = s_ptr[tid + 1]; }
    T acc = T(0);
    for (int32_t base = s0; base < e0; base += kTile) {
      const int32_t tend = min(e0, base + kTile);
#pragma unroll
      for (int j = 0; j < kItems; ++j) {
        const int32_t k = base + j * kBlock + tid;
        if (k < tend) s_prod[k - base] = mul_rn(vals[k], __ldg(p + indices[k]));
      }
      __syncthreads();
      if (tid < nr) {
        const int32_t lo = max(my_s, base), hi = min(my_e, tend);
        for (int32_t k = lo; k < hi; ++k) acc = add_rn(acc, s_prod[k - base]);
      }
      __syncthreads();
    }
    Acc3<T> a{T(0), T(0), T(0)};
    if (tid < nr) {
      q[r0 + tid] = acc;
      a.a = p[r0 + tid] * acc;
    }
    Acc3<T> tot;
    if (sys_reduce(pv, partials, b, s, a, tot) && tid == 0) {
      const T pap = tot.a;
      if (pap <= T(0)) {
        st.status[s] = 1;
        st.message[s] = MSG_NOT_PD;
        atomicSub(pv.ctl + 3, 1);
      } else {
        st.alpha[s] = st.rz_old[s] / pap;
      }
    }
    __syncthreads();
  }
}

// x += alpha p; r -= alpha q; z = dinv r; ||r||, r.z; convergence and beta
template <typename T>
__global__ void __launch_bounds__(kBlock) kb_update(PlanView pv, T* x, T* r, const T* __restrict__ p,
                                                     const T* __restrict__ q, const T* __restrict__ dinv,
                                                     T* partials, SysState<T> st) {
  const int cur = pv.ctl[0];
  const int cnt = pv.ctl[1 + cur];
  const int32_t* list = pv.lists + (int64_t)cur * pv.nblocks;
  for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
    const int b = list[w];
    const int s = pv.blk_sys[b];
    if (st.status[s]) continue;  // uniform across the block
    const int64_t row = pv.blk_row0[b] + threadIdx.x;
    Acc3<T> a{T(0), T(0), T(0)};
    if (threadIdx.x < pv.blk_nrows[b]) {
      const T al = st.alpha[s];
      x[row] = add_rn(x[row], mul_rn(al, p[row]));
      const T ri = sub_rn(r[row], mul_rn(al, q[row]));
      r[row] = ri;
      a.a = ri * ri;
      a.b = ri * mul_rn(ri, dinv[row]);
    }
    Acc3<T> tot;
    if (sys_reduce(pv, partials, b, s, a, tot) && threadIdx.x == 0) {
      const T rn = sqrt(tot.a);
      st.rnorm[s] = rn;
      if (rn <= st.tol[s]) {
        st.status[s] = 1;
        st.converged[s] = 1;
        st.message[s] = MSG_CONVERGED;
        st.iterations[s] += 1;
        atomicSub(pv.ctl + 3, 1);
      } else {
        st.beta[s] = tot.b / st.rz_old[s];
        st.rz_old[s] = tot.b;
      }
    }
    __syncthreads();
  }
}

// p = dinv r + beta p; per-system iteration count and max_iter
template <typename T>
__global__ void __launch_bounds__(kBlock) kb_pupdate(PlanView pv, T* p, const T* __restrict__ r,
                                                      const T* __restrict__ dinv, T* partials,
                                                      SysState<T> st) {
  const int cur = pv.ctl[0];
  const int cnt = pv.ctl[1 + cur];
  const int32_t* list = pv.lists + (int64_t)cur * pv.nblocks;
  for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
    const int b = list[w];
    const int s = pv.blk_sys[b];
    if (st.status[s]) continue;
    const int64_t row = pv.blk_row0[b] + threadIdx.x;
    if (threadIdx.x < pv.blk_nrows[b]) p[row] = add_rn(mul_rn(r[row], dinv[row]), mul_rn(st.beta[s], p[row]));
    Acc3<T> a{T(0), T(0), T(0)}, tot;
    if (sys_reduce(pv, partials, b, s, a, tot) && threadIdx.x == 0) {
      st.iterations[s] += 1;
      if (st.iterations[s] >= st.max_iter) {
        st.status[s] = 1;
        st.message[s] = MSG_MAX_ITER;
        atomicSub(pv.ctl + 3, 1);
      }
    }
    __syncthreads();
  }
}

// drop the blocks of finished systems; re-arm the loop condition
template <typename T>
__global__ void __launch_bounds__(kBlock) kb_compact(PlanView pv, SysState<T> st) {
  const int cur = pv.ctl[0];
  const int nxt = cur ^ 1;
  const int cnt = pv.ctl[1 + cur];
  const int32_t* list = pv.lists + (int64_t)cur * pv.nblocks;
  int32_t* out = pv.lists + (int64_t)nxt * pv.nblocks;
  for (int w = blockIdx.x * kBlock + threadIdx.x; w < cnt; w += gridDim.x * kBlock) {
    const int b = list[w];
    if (!st.status[pv.blk_sys[b]]) out[atomicAdd(pv.ctl + 1 + nxt, 1)] = b;
  }
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd((unsigned*)(pv.ctl + 6), 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    pv.ctl[6] = 0;
    pv.ctl[0] = nxt;
    pv.ctl[1 + cur] = 0;
    if (pv.ctl[4] > 0) pv.ctl[4] -= 1;
    const bool more = pv.ctl[3] > 0 && pv.ctl[4] > 0;
    if (pv.ctl[5]) cudaGraphSetConditional((cudaGraphConditionalHandle)*pv.cond, more ? 1u : 0u);
  }
}

// ---------------------------------------------------------------- setup
// z = dinv r, p = z; rz, ||b||, ||r|| per system; tolerance
template <typename T>
__global__ void __launch_bounds__(kBlock) kb_setup(PlanView pv, const T* __restrict__ b,
                                                    const T* __restrict__ r, const T* __restrict__ dinv,
                                                    T* p, T* partials, SysState<T> st, T rtol, T atol) {
  const int cur = pv.ctl[0];
  const int cnt = pv.ctl[1 + cur];
  const int32_t* list = pv.lists + (int64_t)cur * pv.nblocks;
  for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
    const int bk = list[w];
    const int s = pv.blk_sys[bk];
    const int64_t row = pv.blk_row0[bk] + threadIdx.x;
    Acc3<T> a{T(0), T(0), T(0)};
    if (threadIdx.x < pv.blk_nrows[bk]) {
      const T ri = r[row];
      const T zi = mul_rn(ri, dinv[row]);
      p[row] = zi;
      a.a = ri * zi;
      a.b = b[row] * b[row];
      a.c = ri * ri;
    }
    Acc3<T> tot;
    if (sys_reduce(pv, partials, bk, s, a, tot) && threadIdx.x == 0) {
      st.rz_old[s] = tot.a;
      st.tol[s] = fmax(atol, rtol * sqrt(tot.b));
      st.rnorm[s] = sqrt(tot.c);
      if (st.max_iter == 0) {
        st.status[s] = 1;
        st.message[s] = MSG_MAX_ITER;
        atomicSub(pv.ctl + 3, 1);
      }
    }
    __syncthreads();
  }
}

// FP64 true residual norms per system: rr_s = ||b - A x||^2, bb_s = ||b||^2
__global__ void __launch_bounds__(kBlock) kb_norms64(PlanView pv, const double* __restrict__ b,
                                                      const double* __restrict__ r, double* partials,
                                                      double* rr, double* bb) {
  for (int64_t w = blockIdx.x; w < pv.nblocks; w += gridDim.x) {
    const int bk = (int)w;
    const int s = pv.blk_sys[bk];
    const int64_t row = pv.blk_row0[bk] + threadIdx.x;
    Acc3<double> a{0, 0, 0};
    if (threadIdx.x < pv.blk_nrows[bk]) {
      a.a = r[row] * r[row];
      a.b = b[row] * b[row];
    }
    Acc3<double> tot;
    if (sys_reduce(pv, partials, bk, s, a, tot) && threadIdx.x == 0) {
      rr[s] = tot.a;
      bb[s] = tot.b;
    }
    __syncthreads();
  }
}

// scale residuals of active systems into the FP32 right-hand side
__global__ void kb_scale_down(const int32_t* __restrict__ row_sys, int64_t n, const double* __restrict__ r,
                              const double* __restrict__ rr, const int* __restrict__ active, float* r32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = row_sys[i];
    r32[i] = active[s] ? (float)(r[i] * (1.0 / sqrt(rr[s]))) : 0.0f;
  }
}

__global__ void kb_accumulate(const int32_t* __restrict__ row_sys, int64_t n, double* x,
                              const float* __restrict__ d, const double* __restrict__ rr,
                              const int* __restrict__ active) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = row_sys[i];
    if (active[s]) x[i] = x[i] + sqrt(rr[s]) * (double)d[i];
  }
}

__global__ void kb_row_sys(const int32_t* __restrict__ blk_sys, const int32_t* __restrict__ blk_row0,
                           const int32_t* __restrict__ blk_nrows, int64_t nblocks, int32_t* row_sys) {
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x)
    if (threadIdx.x < blk_nrows[b]) row_sys[blk_row0[b] + threadIdx.x] = blk_sys[b];
}

// initial active list: blocks of systems flagged active
__global__ void kb_init_list(PlanView pv, const int* __restrict__ active) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < pv.nblocks; b += (int64_t)gridDim.x * blockDim.x)
    if (active[pv.blk_sys[b]]) pv.lists[atomicAdd(pv.ctl + 1, 1)] = (int32_t)b;
}

__global__ void kb_jacobi32(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const float* __restrict__ vals, int64_t n, float* dinv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float d = 0.0f;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
      if (idx[k] == (int32_t)i) { d = vals[k]; break; }
    dinv[i] = 1.0f / d;
  }
}

PlanView view(const BatchPlan& p) {
  return PlanView{p.blk_sys, p.blk_row0, p.blk_nrows, p.sys_fb, p.sys_nb, p.lists, p.ctl,
                  p.sys_ticket, p.nblocks, p.cond};
}

void plan_free(BatchPlan& p) {
  dev_free(p.blk_sys); dev_free(p.blk_row0); dev_free(p.blk_nrows); dev_free(p.sys_fb);
  dev_free(p.sys_nb); dev_free(p.lists); dev_free(p.ctl); dev_free(p.sys_ticket);
  dev_free(p.partials); dev_free(p.cond);
  p = BatchPlan{};
}

int plan_build(sx_ctx ctx, const std::vector<int64_t>& sys_ptr, BatchPlan& p) {
  const int64_t S = (int64_t)sys_ptr.size() - 1;
  std::vector<int32_t> bs, br, bn, fb(S), nb(S);
  for (int64_t s = 0; s < S; ++s) {
    fb[s] = (int32_t)bs.size();
    for (int64_t r = sys_ptr[s]; r < sys_ptr[s + 1]; r += kBlock) {
      bs.push_back((int32_t)s);
      br.push_back((int32_t)r);
      bn.push_back((int32_t)std::min<int64_t>(kBlock, sys_ptr[s + 1] - r));
    }
    nb[s] = (int32_t)bs.size() - fb[s];
  }
  p.nsys = S;
  p.nblocks = (int64_t)bs.size();
  p.nrows = sys_ptr[S];
  const size_t B = std::max<int64_t>(p.nblocks, 1), SS = std::max<int64_t>(S, 1);
  SX_CHECK(dev_alloc((void**)&p.blk_sys, B * 4));
  SX_CHECK(dev_alloc((void**)&p.blk_row0, B * 4));
  SX_CHECK(dev_alloc((void**)&p.blk_nrows, B * 4));
  SX_CHECK(dev_alloc((void**)&p.sys_fb, SS * 4));
  SX_CHECK(dev_alloc((void**)&p.sys_nb, SS * 4));
  SX_CHECK(dev_alloc((void**)&p.lists, 2 * B * 4));
  SX_CHECK(dev_alloc((void**)&p.ctl, 16 * 4));
  SX_CHECK(dev_alloc((void**)&p.sys_ticket, SS * 4));
  SX_CHECK(dev_alloc(&p.partials, B * 3 * 8));
  SX_CHECK(dev_alloc((void**)&p.cond, 8));
  if (p.nblocks) {
    SX_CUDA(cudaMemcpy(p.blk_sys, bs.data(), p.nblocks * 4, cudaMemcpyHostToDevice));
    SX_CUDA(cudaMemcpy(p.blk_row0, br.data(), p.nblocks * 4, cudaMemcpyHostToDevice));
    SX_CUDA(cudaMemcpy(p.blk_nrows, bn.data(), p.nblocks * 4, cudaMemcpyHostToDevice));
  }
  if (S) {
    SX_CUDA(cudaMemcpy(p.sys_fb, fb.data(), S * 4, cudaMemcpyHostToDevice));
    SX_CUDA(cudaMemcpy(p.sys_nb, nb.data(), S * 4, cudaMemcpyHostToDevice));
  }
  SX_CUDA(cudaMemset(p.sys_ticket, 0, SS * 4));
  SX_CUDA(cudaMemset(p.ctl, 0, 16 * 4));
  return SX_OK;
}

// Batched FP32 (or FP64) Jacobi-PCG on the systems with active[s] != 0,
// solving A d = rhs from d = 0.  Per-system results into st.
template <typename T>
int batched_cg_core(sx_ctx ctx, const DevCsr& A, const T* dinv, BatchPlan& plan, const int* d_active,
                    int n_active, const T* rhs, T* d, T* r, T* p, T* q, SysState<T>& st, double rtol,
                    double atol, unsigned long long max_iter, uint64_t* launches_out) {
  const int64_t n = A.nrows;
  const PlanView pv = view(plan);
  const int grid = ctx->num_sms * 8;
  // reset control block and the initial active list
  int hctl[16];
  std::memset(hctl, 0, sizeof(hctl));
  hctl[3] = n_active;
  hctl[4] = (int)4096;  // budget per graph launch
  SX_CUDA(cudaMemcpyAsync(plan.ctl, hctl, sizeof(hctl), cudaMemcpyHostToDevice, ctx->stream));
  kb_init_list<<<vec_grid(ctx, plan.nblocks), kBlock, 0, ctx->stream>>>(pv, d_active);
  // d = 0; r = rhs (b - A*0)
  SX_CUDA(cudaMemsetAsync(d, 0, n * sizeof(T), ctx->stream));
  SX_CUDA(cudaMemcpyAsync(r, rhs, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
  kb_setup<T><<<grid, kBlock, 0, ctx->stream>>>(pv, rhs, r, dinv, p, (T*)plan.partials, st, (T)rtol, (T)atol);
  ctx->launches += 2;
  auto body = [&]() -> int {
    kb_spmv_pap<T><<<grid, kBlock, 0, ctx->stream>>>(pv, A.indptr, A.indices, (const T*)A.vals, p, q,
                                                    (T*)plan.partials, st);
    kb_update<T><<<grid, kBlock, 0, ctx->stream>>>(pv, d, r, p, q, dinv, (T*)plan.partials, st);
    kb_pupdate<T><<<grid, kBlock, 0, ctx->stream>>>(pv, p, r, dinv, (T*)plan.partials, st);
    kb_compact<T><<<ctx->num_sms * 2, kBlock, 0, ctx->stream>>>(pv, st);
    ctx->launches += 4;
    SX_CUDA(cudaGetLastError());
    return SX_OK;
  };
  // graph: WHILE(cond) { body }
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaGraphConditionalHandle h = 0;
  bool graph_ok = false;
  do {
    if (cudaGraphCreate(&g, 0) != cudaSuccess) break;
    if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) break;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) != cudaSuccess) break;
    cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(ctx->stream, bodyg, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal) != cudaSuccess) break;
    const uint64_t before = ctx->launches;
    int rc = body();
    cudaGraph_t cap = nullptr;
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &cap);
    ctx->launches = before;
    if (rc != SX_OK || ce != cudaSuccess) break;
    if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) break;
    graph_ok = true;
  } while (0);
  cudaGetLastError();
  unsigned long long hcond = (unsigned long long)h;
  SX_CUDA(cudaMemcpyAsync(plan.cond, &hcond, 8, cudaMemcpyHostToDevice, ctx->stream));
  int rc = SX_OK;
  for (int guard = 0; guard < 1000000; ++guard) {
    int hc[16];
    SX_CUDA(cudaMemcpyAsync(hc, plan.ctl, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hc[3] <= 0) break;
    int refill[2] = {4096, graph_ok ? 1 : 0};
    SX_CUDA(cudaMemcpyAsync(plan.ctl + 4, refill, sizeof(refill), cudaMemcpyHostToDevice, ctx->stream));
    if (graph_ok) {
      SX_CUDA(cudaGraphLaunch(ge, ctx->stream));
      *launches_out += 4ull * 4096ull;  // upper bound; refined below
    } else {
      for (int k = 0; k < 32; ++k)
        if ((rc = body())) break;
      if (rc) break;
    }
  }
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  return rc;
}

}  // namespace
}  // namespace sx

using namespace sx;

extern "C" {

void sx_batched_options_default(sx_batched_options* o) {
  o->max_iter = 10000;
  o->rtol = 1e-8;
  o->atol = 0.0;
  o->inner_rtol = 1e-4;
  o->max_outer = 30;
}

int sx_batched_pcg(sx_ctx ctx, sx_op a64, sx_op a32, const int64_t* sys_ptr, uint64_t nsys,
                   const double* b, double* x, const sx_batched_options* opt, sx_mem mem,
                   sx_batched_result* per_system, sx_batched_summary* summary) {
  if (!ctx || !a64 || !sys_ptr) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a64->kind != SX_OP_CSR || a64->dtype != SX_F64)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: needs an FP64 CSR matrix");
  if (a64->nrows != a64->ncols)
    return set_error(SX_ERR_VALUE, "Value error: Matrix must be square for CG solver");
  if (a32 && (a32->kind != SX_OP_CSR || a32->dtype != SX_F32 || a32->nrows != a64->nrows))
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: a32 must be the FP32 copy of a64");
  sx_batched_options dflt;
  if (!opt) { sx_batched_options_default(&dflt); opt = &dflt; }
  std::vector<int64_t> sp(sys_ptr, sys_ptr + nsys + 1);
  if (sp[0] != 0 || sp[nsys] != a64->nrows)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a64->nrows) + ", found " +
                         std::to_string(sp[nsys]),
                     (uint64_t)a64->nrows, (uint64_t)sp[nsys]);
  for (uint64_t s = 0; s < nsys; ++s)
    if (sp[s + 1] < sp[s]) return set_error(SX_ERR_VALUE, "Value error: system offsets must be non-decreasing");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = a64->nrows;
  const int64_t S = (int64_t)nsys;
  sx_op own32 = nullptr;
  BatchPlan plan;
  double *db = nullptr, *dx = nullptr, *dr = nullptr, *rr = nullptr, *bb = nullptr;
  float *r32 = nullptr, *d32 = nullptr, *rw = nullptr, *pw = nullptr, *qw = nullptr, *dinv = nullptr;
  int32_t* row_sys = nullptr;
  int* active = nullptr;
  SysState<float> st{};
  void* stbuf = nullptr;
  int rc = SX_OK;
  std::vector<uint64_t> inner_total(S, 0);
  std::vector<double> rel(S, 0.0);
  std::vector<int> conv(S, 0);
  uint64_t outer = 0, launches = 0;
  const uint64_t l0 = ctx->launches;
  do {
    if (!a32) {
      if ((rc = sx_csr_astype(ctx, a64, SX_F32, &own32))) break;
      a32 = own32;
    }
    if ((rc = plan_build(ctx, sp, plan))) break;
    const size_t nb = std::max<int64_t>(n, 1), sb = std::max<int64_t>(S, 1);
    if ((rc = dev_alloc((void**)&db, nb * 8))) break;
    if ((rc = dev_alloc((void**)&dx, nb * 8))) break;
    if ((rc = dev_alloc((void**)&dr, nb * 8))) break;
    if ((rc = dev_alloc((void**)&rr, sb * 8))) break;
    if ((rc = dev_alloc((void**)&bb, sb * 8))) break;
    if ((rc = dev_alloc((void**)&r32, nb * 4))) break;
    if ((rc = dev_alloc((void**)&d32, nb * 4))) break;
    if ((rc = dev_alloc((void**)&rw, nb * 4))) break;
    if ((rc = dev_alloc((void**)&pw, nb * 4))) break;
    if ((rc = dev_alloc((void**)&qw, nb * 4))) break;
    if ((rc = dev_alloc((void**)&dinv, nb * 4))) break;
    if ((rc = dev_alloc((void**)&row_sys, nb * 4))) break;
    if ((rc = dev_alloc((void**)&active, sb * 4))) break;
    // per-system state arrays: 5 floats, 3 ints, 1 u64 per system
    if ((rc = dev_alloc(&stbuf, sb * (5 * 4 + 3 * 4 + 8) + 256))) break;
    {
      char* pb = (char*)stbuf;
      st.iterations = (unsigned long long*)pb; pb += sb * 8;
      st.rz_old = (float*)pb; pb += sb * 4;
      st.alpha = (float*)pb; pb += sb * 4;
      st.beta = (float*)pb; pb += sb * 4;
      st.rnorm = (float*)pb; pb += sb * 4;
      st.tol = (float*)pb; pb += sb * 4;
      st.status = (int*)pb; pb += sb * 4;
      st.message = (int*)pb; pb += sb * 4;
      st.converged = (int*)pb; pb += sb * 4;
      st.max_iter = opt->max_iter;
    }
    const cudaMemcpyKind kin = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyAsync(db, b, n * 8, kin, ctx->stream);
    cudaMemsetAsync(dx, 0, n * 8, ctx->stream);
    const int g = vec_grid(ctx, n);
    kb_jacobi32<<<g, kBlock, 0, ctx->stream>>>(a32->csr.indptr, a32->csr.indices,
                                                (const float*)a32->csr.vals, n, dinv);
    kb_row_sys<<<ctx->num_sms * 8, kBlock, 0, ctx->stream>>>(plan.blk_sys, plan.blk_row0, plan.blk_nrows,
                                                             plan.nblocks, row_sys);
    ctx->launches += 2;
    const PlanView pv = view(plan);
    std::vector<double> hrr(S), hbb(S);
    std::vector<int> hact(S);
    std::vector<unsigned long long> hit(S);
    while (true) {
      // FP64 residual and per-system norms
      if ((rc = launch_csr<double>(ctx, a64->csr, dx, dr, EpiResid<double>{db}))) break;
      kb_norms64<<<ctx->num_sms * 8, kBlock, 0, ctx->stream>>>(pv, db, dr, (double*)plan.partials, rr, bb);
      ctx->launches++;
      SX_CUDA(cudaMemcpyAsync(hrr.data(), rr, S * 8, cudaMemcpyDeviceToHost, ctx->stream));
      SX_CUDA(cudaMemcpyAsync(hbb.data(), bb, S * 8, cudaMemcpyDeviceToHost, ctx->stream));
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      int n_act = 0;
      for (int64_t s = 0; s < S; ++s) {
        const double rn = std::sqrt(hrr[s]), bn = std::sqrt(hbb[s]);
        rel[s] = bn > 0 ? rn / bn : rn;
        const bool done = rn <= std::max(opt->atol, opt->rtol * bn);
        conv[s] = done ? 1 : 0;
        hact[s] = (!done && outer < opt->max_outer && sp[s + 1] > sp[s]) ? 1 : 0;
        n_act += hact[s];
      }
      if (n_act == 0) break;
      SX_CUDA(cudaMemcpyAsync(active, hact.data(), S * 4, cudaMemcpyHostToDevice, ctx->stream));
      SX_CUDA(cudaMemsetAsync(stbuf, 0, sb * (5 * 4 + 3 * 4 + 8), ctx->stream));
      kb_scale_down<<<g, kBlock, 0, ctx->stream>>>(row_sys, n, dr, rr, active, r32);
      ctx->launches++;
      // inactive systems start finished so the kernels never visit them
      std::vector<int> hstat(S);
      for (int64_t s = 0; s < S; ++s) hstat[s] = hact[s] ? 0 : 1;
      SX_CUDA(cudaMemcpyAsync(st.status, hstat.data(), S * 4, cudaMemcpyHostToDevice, ctx->stream));
      if ((rc = batched_cg_core<float>(ctx, a32->csr, dinv, plan, active, n_act, r32, d32, rw, pw, qw, st,
                                       opt->inner_rtol, 0.0, opt->max_iter, &launches))) break;
      SX_CUDA(cudaMemcpyAsync(hit.data(), st.iterations, S * 8, cudaMemcpyDeviceToHost, ctx->stream));
      kb_accumulate<<<g, kBlock, 0, ctx->stream>>>(row_sys, n, dx, d32, rr, active);
      ctx->launches++;
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int64_t s = 0; s < S; ++s)
        if (hact[s]) inner_total[s] += hit[s];
      ++outer;
    }
    if (rc) break;
    const cudaMemcpyKind kout = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaMemcpyAsync(x, dx, n * 8, kout, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "batched solution copy", __FILE__, __LINE__);
  } while (0);
  dev_free(db); dev_free(dx); dev_free(dr); dev_free(rr); dev_free(bb); dev_free(r32); dev_free(d32);
  dev_free(rw); dev_free(pw); dev_free(qw); dev_free(dinv); dev_free(row_sys); dev_free(active);
  dev_free(stbuf);
  plan_free(plan);
  if (own32) destroy_op_internal(own32);
  if (rc != SX_OK) return rc;
  uint64_t nconv = 0, maxit = 0, totit = 0;
  double worst = 0.0;
  for (int64_t s = 0; s < S; ++s) {
    if (per_system) {
      per_system[s].inner_iterations = inner_total[s];
      per_system[s].rel_residual = rel[s];
      per_system[s].converged = conv[s];
    }
    nconv += conv[s];
    maxit = std::max<uint64_t>(maxit, inner_total[s]);
    totit += inner_total[s];
    worst = std::max(worst, rel[s]);
  }
  if (summary) {
    summary->outer_iterations = outer;
    summary->converged_systems = nconv;
    summary->max_inner_iterations = maxit;
    summary->total_inner_iterations = totit;
    summary->worst_rel_residual = worst;
    summary->kernel_launches = (ctx->launches - l0) + launches;
  }
  return clear_error();
}

}  // extern "C"
