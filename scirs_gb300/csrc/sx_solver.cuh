// Shared machinery of the device Krylov solvers: the device-side loop
// control, fused elementwise preconditioners, the per-context workspace and
// graph cache, and the WHILE-graph loop runner.  Every scalar of a solver's
// recurrence lives in a device-side state struct whose first member is
// LoopCtl; the last kernel of an iteration re-arms the graph's condition.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"

namespace sx {

enum : int { ST_RUNNING = 0, ST_DONE = 1 };
enum : int { PK_NONE = 0, PK_DIAG = 1, PK_SCALED = 2, PK_GENERAL = 3 };
constexpr unsigned kBudget = 4096;

// Elementwise preconditioners fused into the vector updates.
template <typename T>
struct PrecFused {
  int kind = PK_NONE;
  const T* d = nullptr;
  T s = T(1);
  __device__ __forceinline__ T apply(int64_t i, T r) const {
    if (kind == PK_DIAG) return mul_rn(r, d[i]);
    if (kind == PK_SCALED) return mul_rn(r, s);
    return r;
  }
};

static int prec_kind(sx_op m) {
  if (!m) return PK_NONE;
  switch (m->kind) {
    case SX_OP_IDENTITY: return PK_NONE;
    case SX_OP_DIAGONAL:
    case SX_OP_JACOBI: return PK_DIAG;
    case SX_OP_SCALED_IDENTITY: return PK_SCALED;
    default: return PK_GENERAL;
  }
}

template <typename T>
static PrecFused<T> prec_fused(sx_op m) {
  PrecFused<T> p;
  p.kind = prec_kind(m);
  if (p.kind == PK_DIAG) p.d = (const T*)m->diag;
  if (p.kind == PK_SCALED) p.s = (T)m->scale;
  return p;
}

__device__ __forceinline__ void set_cond(int use, cudaGraphConditionalHandle h, unsigned v) {
  if (use) cudaGraphSetConditional(h, v);
}

template <typename T>
__device__ __forceinline__ T eps_of() { return sizeof(T) == 8 ? (T)2.220446049250313e-16 : (T)1.1920928955078125e-07f; }

// Loop control shared by every solver state (first member of each state):
// the host rewrites only the tail fields (use_cond .. cond) between graph
// launches; everything else is owned by the device.
struct LoopCtl {
  unsigned long long iterations, max_iter;
  int status, message, converged, use_cond;
  unsigned int budget, pad;
  cudaGraphConditionalHandle cond;
};
constexpr size_t kCtlTail = offsetof(LoopCtl, use_cond);

// Epilogue that stores A x but is skipped once the solve has ended.
template <typename T, class S>
struct EpiSkip {
  const S* st;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};


// ================================================================ infra
struct GraphEntry {
  uint64_t key[8];
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle cond = 0;
  int kernels_per_iter = 0;
};

struct SolverCache {
  void* ws = nullptr;
  size_t ws_bytes = 0;
  void* state = nullptr;  // device state block
  std::vector<GraphEntry> graphs;
};

static SolverCache* cache_of(sx_ctx ctx) {
  if (!ctx->solver_cache) ctx->solver_cache = new SolverCache();
  return (SolverCache*)ctx->solver_cache;
}

static void drop_graphs(SolverCache* c) {
  for (auto& g : c->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  c->graphs.clear();
}


constexpr size_t kStateBytes = 4096;

static int ws_get(sx_ctx ctx, size_t bytes, void** ws, void** state) {
  SolverCache* c = cache_of(ctx);
  if (bytes > c->ws_bytes) {
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
    drop_graphs(c);  // graphs captured against the old workspace are stale
    dev_free(c->ws);
    c->ws = nullptr;
    c->ws_bytes = 0;
    SX_CHECK(dev_alloc(&c->ws, bytes));
    c->ws_bytes = bytes;
  }
  if (!c->state) SX_CHECK(dev_alloc(&c->state, kStateBytes));
  *ws = c->ws;
  *state = c->state;
  return SX_OK;
}

static GraphEntry* graph_find(sx_ctx ctx, const uint64_t key[8]) {
  SolverCache* c = cache_of(ctx);
  for (auto& g : c->graphs)
    if (std::memcmp(g.key, key, sizeof(g.key)) == 0) return &g;
  return nullptr;
}

// graph = WHILE(cond) { body }, body captured from `record` (one iteration).
template <class Rec>
static int graph_build(sx_ctx ctx, const uint64_t key[8], Rec record, GraphEntry** out) {
  SolverCache* c = cache_of(ctx);
  if (c->graphs.size() >= 16) drop_graphs(c);
  GraphEntry e;
  std::memcpy(e.key, key, sizeof(e.key));
  SX_CUDA(cudaGraphCreate(&e.graph, 0));
  SX_CUDA(cudaGraphConditionalHandleCreate(&e.cond, e.graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = e.cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  SX_CUDA(cudaGraphAddNode(&node, e.graph, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  SX_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal));
  const uint64_t before = ctx->launches;
  int rc = record();
  cudaGraph_t captured = nullptr;
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &captured);
  e.kernels_per_iter = (int)(ctx->launches - before);
  ctx->launches = before;
  cudaError_t ie = cudaSuccess;
  if (rc == SX_OK && ce == cudaSuccess) ie = cudaGraphInstantiate(&e.exec, e.graph, 0);
  if (rc != SX_OK || ce != cudaSuccess || ie != cudaSuccess) {
    cudaGraphDestroy(e.graph);
    cudaGetLastError();
    // a graph whose programmatic launches the CUDA driver will not capture or
    // instantiate: once more with plain launches for this context
    if (ctx->pdl && (ce != cudaSuccess || ie != cudaSuccess)) {
      ctx->pdl = false;
      clear_error();
      return graph_build(ctx, key, record, out);
    }
    if (rc != SX_OK) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    return cuda_fail(ie, "cudaGraphInstantiate", __FILE__, __LINE__);
  }
  c->graphs.push_back(e);
  *out = &c->graphs.back();
  return SX_OK;
}

// host callbacks cannot run inside a captured graph, also when they sit
// inside a sum or a product
static bool op_graphable(sx_op op) {
  if (!op) return true;
  if (op->kind == SX_OP_HOST) return false;
  return op_graphable(op->left) && op_graphable(op->right);
}

static int check_prec(sx_op a, sx_op m) {
  if (!m) return SX_OK;
  if (m->dtype != a->dtype)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: preconditioner dtype differs");
  if (m->ncols != a->nrows)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(m->ncols) + ", found " +
                         std::to_string(a->nrows),
                     (uint64_t)m->ncols, (uint64_t)a->nrows);
  return SX_OK;
}

static int read_ctl(sx_ctx ctx, const void* d_state, void* h, size_t bytes) {
  void* pin = nullptr;
  SX_CHECK(ctx_pinned(ctx, 2 * kStateBytes, &pin));
  SX_CUDA(cudaMemcpyAsync(pin, d_state, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(h, pin, bytes);
  return SX_OK;
}

static int write_bytes(sx_ctx ctx, void* d_dst, const void* h, size_t bytes) {
  void* pin = nullptr;
  SX_CHECK(ctx_pinned(ctx, 2 * kStateBytes, &pin));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  char* w = (char*)pin + kStateBytes;
  std::memcpy(w, h, bytes);
  SX_CUDA(cudaMemcpyAsync(d_dst, w, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return SX_OK;
}

static int vec_in(sx_ctx ctx, void* dst, const void* src, size_t bytes, sx_mem mem) {
  if (bytes == 0) return SX_OK;
  SX_CUDA(cudaMemcpyAsync(dst, src, bytes,
                          mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          ctx->stream));
  return SX_OK;
}
static int vec_out(sx_ctx ctx, void* dst, const void* src, size_t bytes, sx_mem mem) {
  if (bytes == 0) return SX_OK;
  SX_CUDA(cudaMemcpyAsync(dst, src, bytes,
                          mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          ctx->stream));
  return SX_OK;
}

// Rows from which the CG loops run as stream launches rather than a captured
// graph while SpMVs are programmatic: consecutive programmatic launches
// overlap on a stream but not inside a graph's WHILE body (1024^2 Q1 learned
// solve: 102.4 ms on the stream, 106.4 ms as a graph; small problems keep
// the graph, whose launches cost the host nothing)
constexpr int64_t kStreamLoopRows = int64_t(1) << 18;
static bool loop_as_graph(sx_ctx ctx, int64_t n) { return !(ctx->pdl && n >= kStreamLoopRows); }

// Runs iterations until the state reports the end.  With a graph, one launch
// executes up to kBudget iterations of the captured body; otherwise the same
// body is enqueued in chunks of 32 iterations.
template <class Rec>
static int run_loop(sx_ctx ctx, void* d_state, const uint64_t key[8], bool graphable,
                    Rec record) {
  LoopCtl h;
  SX_CHECK(read_ctl(ctx, d_state, &h, sizeof(h)));
  if (h.status != ST_RUNNING) return SX_OK;
  GraphEntry* g = nullptr;
  // SX_GRAPHS=0 launches the same kernels eagerly (per-kernel profiling)
  const char* env = std::getenv("SX_GRAPHS");
  if (env && env[0] == '0') graphable = false;
  if (graphable) {
    g = graph_find(ctx, key);
    if (!g) {
      int rc = graph_build(ctx, key, record, &g);
      if (rc != SX_OK) g = nullptr;  // fall back to eager launches
    }
  }
  for (int guard = 0;; ++guard) {
    const unsigned long long it0 = h.iterations;
    LoopCtl tail;
    std::memset(&tail, 0, sizeof(tail));
    tail.use_cond = g ? 1 : 0;
    tail.budget = kBudget;
    tail.cond = g ? g->cond : 0;
    SX_CHECK(write_bytes(ctx, (char*)d_state + kCtlTail, (const char*)&tail + kCtlTail,
                         sizeof(LoopCtl) - kCtlTail));
    if (g) {
      SX_CUDA(cudaGraphLaunch(g->exec, ctx->stream));
    } else {
      for (int k = 0; k < 32; ++k) SX_CHECK(record());
    }
    SX_CHECK(read_ctl(ctx, d_state, &h, sizeof(h)));
    if (g) ctx->launches += (uint64_t)g->kernels_per_iter * (h.iterations - it0 + 1);
    if (h.status != ST_RUNNING) break;
    if (h.iterations == it0 && guard > 2)
      return set_error(SX_ERR_ITERATIVE_SOLVER_FAILURE,
                       "Iterative solver failure: device loop made no progress");
  }
  return SX_OK;
}


// Argument checks shared by the solver entry points: a square operator
// (ValueError "Matrix must be square for <name> solver") and b of its size.
static int solver_checks(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, void* x_out,
                         const char* name) {
  if (!ctx || !a) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx/operator");
  if (a->nrows != a->ncols)
    return set_error(SX_ERR_VALUE,
                     std::string("Value error: Matrix must be square for ") + name + " solver");
  if (b_len != (uint64_t)a->nrows)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a->nrows) + ", found " +
                         std::to_string(b_len),
                     (uint64_t)a->nrows, b_len);
  if (a->nrows > 0 && (!b || !x_out))
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null b/x");
  SX_CUDA(cudaSetDevice(ctx->device));
  return SX_OK;
}


}  // namespace sx
