// Krylov solvers of scirs2-sparse on the device (linalg/iterative.rs):
// cg (:40-162), bicgstab (:377-611), gmres (:641-816).
//
// Every scalar of the recurrences lives in a device-side state struct.  The
// reductions of an iteration are fused into the kernel that produces their
// operands (the SpMV epilogue for p.Ap, the vector update for r.r and r.z),
// and the last block of each reduction performs the reference's scalar step
// and its exits (breakdown, convergence, max_iter) in the reference's order.
// Kernels of later steps return at once when the state says the solve has
// ended, so an iteration can be replayed without host involvement: the loop
// body is captured once into a CUDA graph whose conditional WHILE node is
// re-armed by the last kernel of each iteration.  A graph launch runs at most
// `budget` iterations, so the host regains control periodically.

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sx_launch.cuh"
#include "sx_mixed.cuh"
#include "sx_solver.cuh"

namespace sx {

void solver_graphs_drop(sx_ctx ctx) {
  if (ctx->solver_cache) drop_graphs((SolverCache*)ctx->solver_cache);
}

// ===================================================================== CG
template <typename T>
struct CgState {
  LoopCtl c;
  T rz_old, alpha, beta, rnorm, tol, pap, rtol, atol, result_norm;
};

// z = M r, p = z, rz = r.z, ||b||, ||r|| (iterative.rs:82-93)
template <typename T>
struct CgSetup {
  CgState<T>* st;
  const T *b, *r, *z;  // z only for a general preconditioner
  T* p;
  PrecFused<T> pf;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    T ri = r[i];
    T zi = pf.kind == PK_GENERAL ? z[i] : pf.apply(i, ri);
    p[i] = zi;
    a.a += ri * zi;
    a.b += b[i] * b[i];
    a.c += ri * ri;
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rz_old = t.a;
    T bnorm = sqrt(t.b);
    st->tol = fmax(st->atol, st->rtol * bnorm);
    st->rnorm = sqrt(t.c);
    st->result_norm = st->rnorm;
    if (st->c.max_iter == 0) {
      st->c.status = ST_DONE;
      st->c.message = MSG_MAX_ITER;
    }
  }
};

// Ap with pAp fused (iterative.rs:98-111)
template <typename T>
struct EpiCgPap {
  static constexpr bool kBanded = true;
  CgState<T>* st;
  const T* p;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t i, T y, Acc3<T>& a) const { a.a += p[i] * y; }
  __device__ void finish(const Acc3<T>& t) const {
    T pap = t.a;
    st->pap = pap;
    if (pap <= T(0)) {
      st->c.status = ST_DONE;
      st->c.message = MSG_NOT_PD;
      st->result_norm = st->rnorm;
      return;
    }
    st->alpha = st->rz_old / pap;
  }
};

// a + b c: one fused multiply-add in FP64, where GB300's FP64 pipe (two
// lanes per clock per SM) bounds the vector updates; the reference's two
// roundings in FP32
template <typename T>
__device__ __forceinline__ T axpy_rn(T a, T b, T c) {
  if constexpr (sizeof(T) == 8) return fma(b, c, a);
  else return add_rn(a, mul_rn(b, c));
}

// x += alpha p; r -= alpha Ap; ||r||; r.z for a fused M (iterative.rs:113-144)
template <typename T>
struct CgUpdate {
  CgState<T>* st;
  T *x, *r;
  const T *p, *ap;
  PrecFused<T> pf;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  static constexpr bool kVec4 = true;
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T alpha = st->alpha;
    x[i] = axpy_rn(x[i], alpha, p[i]);
    T ri = axpy_rn(r[i], -alpha, ap[i]);
    r[i] = ri;
    a.a += ri * ri;
    if (pf.kind != PK_GENERAL) a.b += ri * pf.apply(i, ri);
  }
  __device__ void elem4(int64_t i, Acc3<T>& a) const {
    const T alpha = st->alpha;
    Vec4<T> xv = ldv4(x + i), pv = ldv4(p + i), rv = ldv4(r + i), qv = ldv4(ap + i);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      xv.v[q] = axpy_rn(xv.v[q], alpha, pv.v[q]);
      rv.v[q] = axpy_rn(rv.v[q], -alpha, qv.v[q]);
      a.a += rv.v[q] * rv.v[q];
    }
    // one branch on the preconditioner per four elements (not a select per
    // element, which evaluates every kind's product)
    if (pf.kind == PK_DIAG) {
      const Vec4<T> dv = ldv4(pf.d + i);
#pragma unroll
      for (int q = 0; q < 4; ++q) a.b += rv.v[q] * mul_rn(rv.v[q], dv.v[q]);
    } else if (pf.kind == PK_SCALED) {
#pragma unroll
      for (int q = 0; q < 4; ++q) a.b += rv.v[q] * mul_rn(rv.v[q], pf.s);
    } else if (pf.kind != PK_GENERAL) {
#pragma unroll
      for (int q = 0; q < 4; ++q) a.b += rv.v[q] * rv.v[q];
    }
    stv4(x + i, xv);
    stv4(r + i, rv);
  }
  __device__ void finish(const Acc3<T>& t) const {
    T rnorm = sqrt(t.a);
    st->rnorm = rnorm;
    if (rnorm <= st->tol) {
      st->c.status = ST_DONE;
      st->c.converged = 1;
      st->c.message = MSG_CONVERGED;
      st->c.iterations += 1;
      st->result_norm = rnorm;
      return;
    }
    if (pf.kind != PK_GENERAL) {
      T rz_new = t.b;
      st->beta = rz_new / st->rz_old;
      st->rz_old = rz_new;
    }
  }
};

// z = M r with r.z and beta fused into the epilogue of the preconditioner
// apply (general M: IC(0), FSAI, learned; iterative.rs:143-144); skipped
// once the solve has ended
template <typename T>
struct EpiCgRz {
  static constexpr bool kBanded = true;
  CgState<T>* st;
  const T* r;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T z) const { return z; }
  __device__ void acc(int64_t i, T z, Acc3<T>& a) const { a.a += r[i] * z; }
  __device__ void finish(const Acc3<T>& t) const {
    st->beta = t.a / st->rz_old;
    st->rz_old = t.a;
  }
};

// p = z + beta p; iteration count; loop condition (iterative.rs:147-152)
template <typename T>
struct CgP {
  CgState<T>* st;
  T* p;
  const T *r, *z;
  PrecFused<T> pf;
  static constexpr bool kReduce = true;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  static constexpr bool kVec4 = true;
  __device__ void elem(int64_t i, Acc3<T>&) const {
    T zi = pf.kind == PK_GENERAL ? z[i] : pf.apply(i, r[i]);
    p[i] = axpy_rn(zi, st->beta, p[i]);
  }
  __device__ void elem4(int64_t i, Acc3<T>&) const {
    const T beta = st->beta;
    Vec4<T> pv = ldv4(p + i);
    Vec4<T> zv;
    if (pf.kind == PK_GENERAL) {
      zv = ldv4(z + i);
    } else {
      zv = ldv4(r + i);
      if (pf.kind == PK_DIAG) {
        const Vec4<T> dv = ldv4(pf.d + i);
#pragma unroll
        for (int q = 0; q < 4; ++q) zv.v[q] = mul_rn(zv.v[q], dv.v[q]);
      } else if (pf.kind == PK_SCALED) {
#pragma unroll
        for (int q = 0; q < 4; ++q) zv.v[q] = mul_rn(zv.v[q], pf.s);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) pv.v[q] = axpy_rn(zv.v[q], beta, pv.v[q]);
    stv4(p + i, pv);
  }
  __device__ void finish(const Acc3<T>&) const {
    st->c.iterations += 1;
    if (st->c.iterations >= st->c.max_iter) {
      st->c.status = ST_DONE;
      st->c.message = MSG_MAX_ITER;
      st->result_norm = st->rnorm;
    }
    if (st->c.budget > 0) st->c.budget -= 1;
    set_cond(st->c.use_cond, st->c.cond,
             (st->c.status == ST_RUNNING && st->c.budget > 0) ? 1u : 0u);
  }
};

// ---- CG in two kernels per iteration (opt-in, sx_ctx_set_cg_recurrence):
// for diagonal preconditioners, A p is carried by the recurrence
// q = A z + beta q instead of a product of A with p, so the p-update folds
// into the SpMV's epilogue and z = D r into the vector update.  Every other
// operation is the reference loop's (iterative.rs:95-151) with the same
// roundings; q differs from A p by the recurrence's rounding.
//   setup  z = D r, p = 0, q = 0, beta = 0, rz, ||b||, ||r||, tol
//   K1     w = A z; p = z + beta p; q = w + beta q; p.q -> alpha
//   K2     x += alpha p; r -= alpha q; ||r|| (convergence); z = D r; r.z -> beta;
//          iteration count, max_iter, graph condition
template <typename T>
struct CgSetupQ {
  CgState<T>* st;
  const T *b, *r;
  T *z, *p;
  PrecFused<T> pf;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T ri = r[i];
    const T zi = pf.apply(i, ri);
    z[i] = zi;
    p[i] = T(0);
    a.a += ri * zi;
    a.b += b[i] * b[i];
    a.c += ri * ri;
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rz_old = t.a;
    st->beta = T(0);
    T bnorm = sqrt(t.b);
    st->tol = fmax(st->atol, st->rtol * bnorm);
    st->rnorm = sqrt(t.c);
    st->result_norm = st->rnorm;
    if (st->c.max_iter == 0) {
      st->c.status = ST_DONE;
      st->c.message = MSG_MAX_ITER;
    }
  }
};

// K1's epilogue: y is q (updated in place), p is updated beside it
template <typename T>
struct EpiCgQ {
  static constexpr bool kBanded = true;
  CgState<T>* st;
  const T* z;
  T *p, *q;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t i, T w) const {
    const T b = st->beta;
    p[i] = axpy_rn(z[i], b, p[i]);
    return axpy_rn(w, b, q[i]);  // stored to q[i]
  }
  __device__ void acc(int64_t i, T qi, Acc3<T>& a) const { a.a += p[i] * qi; }
  __device__ void finish(const Acc3<T>& t) const {
    const T pap = t.a;
    st->pap = pap;
    if (pap <= T(0)) {
      st->c.status = ST_DONE;
      st->c.message = MSG_NOT_PD;
      st->result_norm = st->rnorm;
      return;
    }
    st->alpha = st->rz_old / pap;
  }
};

template <typename T>
struct CgUpdateQ {
  CgState<T>* st;
  T *x, *r, *z;
  const T *p, *q;
  PrecFused<T> pf;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = true;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T alpha = st->alpha;
    x[i] = axpy_rn(x[i], alpha, p[i]);
    const T ri = axpy_rn(r[i], -alpha, q[i]);
    r[i] = ri;
    const T zi = pf.apply(i, ri);
    z[i] = zi;
    a.a += ri * ri;
    a.b += ri * zi;
  }
  __device__ void elem4(int64_t i, Acc3<T>& a) const {
    const T alpha = st->alpha;
    Vec4<T> xv = ldv4(x + i), pv = ldv4(p + i), rv = ldv4(r + i), qv = ldv4(q + i), zv;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      xv.v[k] = axpy_rn(xv.v[k], alpha, pv.v[k]);
      rv.v[k] = axpy_rn(rv.v[k], -alpha, qv.v[k]);
    }
    // one branch on the preconditioner per four elements (a select per
    // element evaluated every kind's product and reloaded D: 2.4x the FP64
    // work on GB300's thin FP64 pipe)
    if (pf.kind == PK_DIAG) {
      const Vec4<T> dv = ldv4(pf.d + i);
#pragma unroll
      for (int k = 0; k < 4; ++k) zv.v[k] = mul_rn(rv.v[k], dv.v[k]);
    } else if (pf.kind == PK_SCALED) {
#pragma unroll
      for (int k = 0; k < 4; ++k) zv.v[k] = mul_rn(rv.v[k], pf.s);
    } else {
      zv = rv;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a.a += rv.v[k] * rv.v[k];
      a.b += rv.v[k] * zv.v[k];
    }
    stv4(x + i, xv);
    stv4(r + i, rv);
    stv4(z + i, zv);
  }
  __device__ void finish(const Acc3<T>& t) const {
    const T rnorm = sqrt(t.a);
    st->rnorm = rnorm;
    if (rnorm <= st->tol) {
      st->c.status = ST_DONE;
      st->c.converged = 1;
      st->c.message = MSG_CONVERGED;
      st->c.iterations += 1;
      st->result_norm = rnorm;
      set_cond(st->c.use_cond, st->c.cond, 0u);
      return;
    }
    st->beta = t.b / st->rz_old;
    st->rz_old = t.b;
    st->c.iterations += 1;
    if (st->c.iterations >= st->c.max_iter) {
      st->c.status = ST_DONE;
      st->c.message = MSG_MAX_ITER;
      st->result_norm = st->rnorm;
    }
    if (st->c.budget > 0) st->c.budget -= 1;
    set_cond(st->c.use_cond, st->c.cond, (st->c.status == ST_RUNNING && st->c.budget > 0) ? 1u : 0u);
  }
};

template <typename T>
static int cg_run(sx_ctx ctx, sx_op a, const void* b, const sx_cg_options* opt, void* x_out,
                  sx_mem mem, sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m = opt->preconditioner;
  SX_CHECK(check_prec(a, m));
  const int pk = prec_kind(m);
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 6, &ws, &dstate));
  T* vb_ = (T*)ws;
  T* B = (T*)((char*)ws + 0 * vb);
  T* X = (T*)((char*)ws + 1 * vb);
  T* R = (T*)((char*)ws + 2 * vb);
  T* P = (T*)((char*)ws + 3 * vb);
  T* AP = (T*)((char*)ws + 4 * vb);
  T* Z = (T*)((char*)ws + 5 * vb);
  (void)vb_;
  CgState<T>* st = (CgState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  CgState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  const PrecFused<T> pf = prec_fused<T>(m);
  // r = b - A x (iterative.rs:78-79)
  SX_CHECK(launch_apply<T>(ctx, a, X, R, EpiResid<T>{B}));
  if (pk == PK_GENERAL)
    SX_CHECK(launch_apply<T>(ctx, m, R, Z, EpiPlain<T>{}));
  const bool recur = ctx->cg_recurrence && pk != PK_GENERAL;
  if (recur) {
    if (n > 0) SX_CUDA(cudaMemsetAsync(AP, 0, n * w, ctx->stream));
    SX_CHECK(launch_vec<T>(ctx, n, CgSetupQ<T>{st, B, R, Z, P, pf}));
  } else {
    SX_CHECK(launch_vec<T>(ctx, n, CgSetup<T>{st, B, R, Z, P, pf}));
  }
  auto body = [&]() -> int {
    if (recur) {
      SX_CHECK(launch_apply<T>(ctx, a, Z, AP, EpiCgQ<T>{st, Z, P, AP}));
      SX_CHECK(launch_vec<T>(ctx, n, CgUpdateQ<T>{st, X, R, Z, P, AP, pf}));
      return SX_OK;
    }
    SX_CHECK(launch_apply<T>(ctx, a, P, AP, EpiCgPap<T>{st, P}));
    SX_CHECK(launch_vec<T>(ctx, n, CgUpdate<T>{st, X, R, P, AP, pf}));
    if (pk == PK_GENERAL) {
      SX_CHECK(launch_apply<T>(ctx, m, R, Z, EpiCgRz<T>{st, R}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, CgP<T>{st, P, R, Z, pf}));
    return SX_OK;
  };
  const uint64_t key[8] = {1, (uint64_t)sizeof(T), a->serial, m ? m->serial : 0,
                           (uint64_t)n, (uint64_t)(uintptr_t)ws, (uint64_t)pk, recur ? 1u : 0u};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m) && loop_as_graph(ctx, n), body));
  SX_CHECK(ic0_health(ctx, m));
  SX_CHECK(ic0_health(ctx, a));
  SX_CHECK(read_ctl(ctx, st, &h, sizeof(h)));
  SX_CHECK(vec_out(ctx, x_out, X, n * w, mem));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (res) {
    res->iterations = h.c.iterations;
    res->residual_norm = (double)h.result_norm;
    res->converged = h.c.converged;
    res->message = h.c.message;
  }
  return SX_OK;
}

// ============================== FP32 CG with FP64 residual replacement
// One FP32 PCG run split into segments (cg_mixed_replace below).  Between
// segments the FP32 iterate is folded into the FP64 solution, the FP64 true
// residual replaces the FP32 one, and the recurrence continues:
// beta = r'.z' / rz_old, p = z' + beta p.

// x64 += x32; x32 = 0
struct IrFold {
  double* x64;
  float* x32;
  static constexpr bool kReduce = false;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<double>&) const {
    x64[i] = x64[i] + (double)x32[i];
    x32[i] = 0.0f;
  }
  __device__ void finish(const Acc3<double>&) const {}
};

// r32 = (float) r64 (and a second copy, the segment's reference vector)
struct IrNarrow {
  const double* r64;
  float *r32, *copy;
  static constexpr bool kReduce = false;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<double>&) const {
    const float v = (float)r64[i];
    r32[i] = v;
    if (copy) copy[i] = v;
  }
  __device__ void finish(const Acc3<double>&) const {}
};

// a new segment: beta from the replaced residual, threshold, counters
__device__ __forceinline__ void ir_restart(CgState<float>* st, float rz, float rr) {
  st->beta = rz / st->rz_old;
  st->rz_old = rz;
  st->rnorm = sqrtf(rr);
  st->result_norm = st->rnorm;
  st->tol = fmaxf(st->atol, st->rtol * st->rnorm);
  st->c.status = ST_RUNNING;
  st->c.converged = 0;
  st->c.message = MSG_CONVERGED;
  st->c.iterations = 0;
}

// r32 = (float) r64 with r.z (fused elementwise M) and r.r
struct IrNarrowRz {
  CgState<float>* st;
  const double* r64;
  float* r32;
  PrecFused<float> pf;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<float>& a) const {
    const float r = (float)r64[i];
    r32[i] = r;
    a.a += r * pf.apply(i, r);
    a.b += r * r;
  }
  __device__ void finish(const Acc3<float>& t) const { ir_restart(st, t.a, t.b); }
};

// r.z and r.r for a general M (z = M r already applied)
struct IrRz {
  CgState<float>* st;
  const float *r, *z;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<float>& a) const {
    a.a += r[i] * z[i];
    a.b += r[i] * r[i];
  }
  __device__ void finish(const Acc3<float>& t) const { ir_restart(st, t.a, t.b); }
};

// p = z + beta p after a replacement (no iteration counted)
struct IrP {
  CgState<float>* st;
  float* p;
  const float *r, *z;
  PrecFused<float> pf;
  static constexpr bool kReduce = false;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<float>&) const {
    const float zi = pf.kind == PK_GENERAL ? z[i] : pf.apply(i, r[i]);
    p[i] = add_rn(zi, mul_rn(st->beta, p[i]));
  }
  __device__ void finish(const Acc3<float>&) const {}
};

// ---- fused FP32 iteration of the residual-replacement loop.  With
// q = A p kept as its own recurrence (A p_new = A z + beta A p_old), the
// p update moves into the SpMV epilogue, and for M = G G^T the x/r update
// moves into the G^T SpMV, whose gathers form r - alpha q on the fly:
//   K1  w = A z;  p = z + beta p;  q = w + beta q;  p.q -> alpha
//   K2  (Jacobi) x += alpha p; r -= alpha q; z = D r; ||r||, r.z -> beta
//   K2  (G G^T) t = G^T (r - alpha q); x += alpha p; r' = r - alpha q; ||r'||
//   K3  (G G^T) z = G t; r'.z -> beta
// r ping-pongs between two buffers (G G^T); a captured body runs two
// iterations, R[0] -> R[1] -> R[0], so every segment starts from R[0].
struct MxState {
  CgState<float> cg;  // first: the loop control sits at offset 0
  int rsel, pad;
};

struct EpiMx1 {
  static constexpr bool kBanded = true;
  CgState<float>* st;
  const float* z;
  float *p, *q;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ float out(int64_t i, float w) const {
    const float b = st->beta;
    p[i] = add_rn(z[i], mul_rn(b, p[i]));
    return add_rn(w, mul_rn(b, q[i]));  // stored to q[i]
  }
  __device__ void acc(int64_t i, float qi, Acc3<float>& a) const { a.a += p[i] * qi; }
  __device__ void out_acc4(int64_t i, const float (&w)[4], float (&o)[4], Acc3<float>& a) const {
    const float b = st->beta;
    const Vec4<float> z4 = ldv4(z + i), p4 = ldv4(p + i), q4 = ldv4(q + i);
    Vec4<float> pn;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      pn.v[j] = add_rn(z4.v[j], mul_rn(b, p4.v[j]));
      o[j] = add_rn(w[j], mul_rn(b, q4.v[j]));
    }
    stv4(p + i, pn);
#pragma unroll
    for (int j = 0; j < 4; ++j) a.a += pn.v[j] * o[j];
  }
  __device__ void finish(const Acc3<float>& t) const {
    st->pap = t.a;
    if (t.a <= 0.0f) {
      st->c.status = ST_DONE;
      st->c.message = MSG_NOT_PD;
      st->result_norm = st->rnorm;
      return;
    }
    st->alpha = st->rz_old / t.a;
  }
};

// end of an iteration: count, max_iter, budget, graph condition
__device__ __forceinline__ void mx_end_iteration(CgState<float>* st) {
  st->c.iterations += 1;
  if (st->c.iterations >= st->c.max_iter) {
    st->c.status = ST_DONE;
    st->c.message = MSG_MAX_ITER;
    st->result_norm = st->rnorm;
  }
  if (st->c.budget > 0) st->c.budget -= 1;
  set_cond(st->c.use_cond, st->c.cond, (st->c.status == ST_RUNNING && st->c.budget > 0) ? 1u : 0u);
}
__device__ __forceinline__ bool mx_converged(CgState<float>* st, float rnorm) {
  st->rnorm = rnorm;
  if (rnorm <= st->tol) {
    st->c.status = ST_DONE;
    st->c.converged = 1;
    st->c.message = MSG_CONVERGED;
    st->c.iterations += 1;
    st->result_norm = rnorm;
    set_cond(st->c.use_cond, st->c.cond, 0u);
    return true;
  }
  return false;
}

// K2 for Jacobi: x, r, z = D r, ||r||, r.z, beta
struct MxJacobiUpdate {
  CgState<float>* st;
  float *x, *r, *z;
  const float *p, *q, *d;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  __device__ void elem(int64_t i, Acc3<float>& a) const {
    const float al = st->alpha;
    x[i] = add_rn(x[i], mul_rn(al, p[i]));
    const float ri = sub_rn(r[i], mul_rn(al, q[i]));
    r[i] = ri;
    const float zi = mul_rn(ri, d[i]);
    z[i] = zi;
    a.a += ri * ri;
    a.b += ri * zi;
  }
  __device__ void finish(const Acc3<float>& t) const {
    if (mx_converged(st, sqrtf(t.a))) return;
    st->beta = t.b / st->rz_old;
    st->rz_old = t.b;
    mx_end_iteration(st);
  }
};

// K2 for G G^T: gathers r - alpha q, updates x and r' in the epilogue
struct GatherMxResid {
  const float *r, *q;
  const CgState<float>* st;
  __device__ __forceinline__ float operator()(const float*, int c) const {
    return sub_rn(__ldg(r + c), mul_rn(st->alpha, __ldg(q + c)));
  }
  // the same values for four aligned columns (the diagonal-layout kernel)
  template <int VEC>
  __device__ __forceinline__ void vec(const float*, int c, float (&o)[VEC]) const {
    float rv[VEC], qv[VEC];
    vload(r + c, rv);
    vload(q + c, qv);
    const float al = st->alpha;
#pragma unroll
    for (int j = 0; j < VEC; ++j) o[j] = sub_rn(rv[j], mul_rn(al, qv[j]));
  }
};
struct EpiMx2 {
  static constexpr bool kBanded = true;
  MxState* ms;
  float* x;
  const float *p, *q, *r;
  float* rn;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return ms->cg.c.status != ST_RUNNING; }
  __device__ float out(int64_t, float t) const { return t; }
  __device__ void acc(int64_t i, float, Acc3<float>& a) const {
    const float al = ms->cg.alpha;
    x[i] = add_rn(x[i], mul_rn(al, p[i]));
    const float ri = sub_rn(r[i], mul_rn(al, q[i]));  // the value the gathers formed
    rn[i] = ri;
    a.a += ri * ri;
  }
  __device__ void out_acc4(int64_t i, const float (&t)[4], float (&o)[4], Acc3<float>& a) const {
    const float al = ms->cg.alpha;
    const Vec4<float> x4 = ldv4(x + i), p4 = ldv4(p + i), r4 = ldv4(r + i), q4 = ldv4(q + i);
    Vec4<float> xn, rv;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      o[j] = t[j];
      xn.v[j] = add_rn(x4.v[j], mul_rn(al, p4.v[j]));
      rv.v[j] = sub_rn(r4.v[j], mul_rn(al, q4.v[j]));
    }
    stv4(x + i, xn);
    stv4(rn + i, rv);
#pragma unroll
    for (int j = 0; j < 4; ++j) a.a += rv.v[j] * rv.v[j];
  }
  __device__ void finish(const Acc3<float>& t) const {
    ms->rsel ^= 1;
    mx_converged(&ms->cg, sqrtf(t.a));
  }
};
// K3 for G G^T: z = G t with r'.z, beta, end of the iteration
struct EpiMx3 {
  static constexpr bool kBanded = true;
  CgState<float>* st;
  const float* rn;
  static constexpr bool kReduce = true;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  __device__ float out(int64_t, float z) const { return z; }
  __device__ void acc(int64_t i, float z, Acc3<float>& a) const { a.a += rn[i] * z; }
  __device__ void out_acc4(int64_t i, const float (&z)[4], float (&o)[4], Acc3<float>& a) const {
    const Vec4<float> r4 = ldv4(rn + i);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      o[j] = z[j];
      a.a += r4.v[j] * z[j];
    }
  }
  __device__ void finish(const Acc3<float>& t) const {
    st->beta = t.a / st->rz_old;
    st->rz_old = t.a;
    mx_end_iteration(st);
  }
};

// a segment start: p = q = 0, beta = 0 (so K1 forms p = z, q = A z), z = D r
// (Jacobi) or the already applied z, r.z, ||r||, threshold
struct MxStart {
  CgState<float>* st;
  const double* r64;  // non-null: r = (float) r64 first
  float *r, *z, *p, *q;
  const float* d;     // Jacobi diagonal, or null (z given)
  bool restart;       // false: first segment (no beta from a previous r.z)
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<float>& a) const {
    float ri = r64 ? (float)r64[i] : r[i];
    if (r64) r[i] = ri;
    float zi;
    if (d) { zi = mul_rn(ri, d[i]); z[i] = zi; }
    else zi = z[i];
    if (!restart) { p[i] = 0.0f; q[i] = 0.0f; }
    a.a += ri * zi;
    a.b += ri * ri;
  }
  __device__ void finish(const Acc3<float>& t) const {
    if (restart) {
      ir_restart(st, t.a, t.b);
    } else {
      st->beta = 0.0f;
      st->rz_old = t.a;
      st->rnorm = sqrtf(t.b);
      st->result_norm = st->rnorm;
      st->tol = fmaxf(st->atol, st->rtol * st->rnorm);
      st->c.status = ST_RUNNING;
      st->c.converged = 0;
      st->c.message = MSG_CONVERGED;
      st->c.iterations = 0;
    }
  }
};

// The fused loop; false (nothing launched) when it does not apply: M must
// be Jacobi or G G^T with both factors fitting the register pipeline.
static int cg_mixed_fused(sx_ctx ctx, sx_op a64, sx_op a32, sx_op m, const double* db, double* dx, double* dr,
                          IrNorms* nrm, const sx_ir_options* opt, uint64_t* outer, uint64_t* inner, double* rel,
                          int* converged, bool* applied) {
  *applied = false;
  const int pk = prec_kind(m);
  const bool jac = pk == PK_DIAG;
  const bool gg = m && m->kind == SX_OP_FSAI;
  if (!jac && !gg) return SX_OK;
  auto fits = [](const DevCsr& c) { return c.monotone && c.max_chunk_nnz + 3 <= kBlock * 12; };
  if (!fits(a32->csr) || (gg && !(fits(m->csr) && fits(m->transpose->csr)))) return SX_OK;
  SX_CHECK(check_prec(a32, m));
  *applied = true;
  using T = float;
  const int64_t n = a64->nrows;
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * sizeof(T), 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 8, &ws, &dstate));
  auto vec = [&](int k) { return (T*)((char*)ws + k * vb); };
  T *X = vec(0), *R[2] = {vec(1), vec(2)}, *P = vec(3), *Q = vec(4), *Z = vec(5), *TW = vec(6);
  MxState* ms = (MxState*)dstate;
  CgState<T>* st = &ms->cg;
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  const T* dinv = jac ? (const T*)m->diag : nullptr;

  auto true_residual = [&](IrNorms& h) -> int {
    SX_CHECK(launch_csr<double, EpiIrResid, true>(ctx, a64->csr, dx, dr, EpiIrResid{db, nrm}));
    SX_CHECK(read_ctl(ctx, nrm, &h, sizeof(h)));
    return SX_OK;
  };
  IrNorms h;
  SX_CHECK(true_residual(h));
  const double bnorm = std::sqrt(h.bb);
  double rnorm = std::sqrt(h.rr);
  *rel = bnorm > 0 ? rnorm / bnorm : rnorm;
  if (rnorm <= opt->tol * bnorm) {
    *converged = 1;
    return SX_OK;
  }
  const double delta = (opt->replace_factor > 0.0 && opt->replace_factor < 1.0) ? opt->replace_factor : 0.1;
  MxState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.cg.c.max_iter = opt->max_inner;
  hs.cg.rtol = (T)delta;
  hs.cg.atol = (T)(0.5 * opt->tol * bnorm);
  SX_CHECK(write_bytes(ctx, ms, &hs, sizeof(hs)));
  if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * sizeof(T), ctx->stream));
  // first segment
  if (jac) {
    SX_CHECK(launch_vec<T>(ctx, n, MxStart{st, dr, R[0], Z, P, Q, dinv, false}));
  } else {
    SX_CHECK(launch_vec<double>(ctx, n, IrNarrow{dr, R[0], nullptr}));
    SX_CHECK(launch_apply<T>(ctx, m, R[0], Z, EpiPlain<T>{}));
    SX_CHECK(launch_vec<T>(ctx, n, MxStart{st, nullptr, R[0], Z, P, Q, nullptr, false}));
  }
  auto k1 = [&]() { return launch_apply<T>(ctx, a32, Z, Q, EpiMx1{st, Z, P, Q}); };
  auto body = [&]() -> int {
    if (jac) {
      SX_CHECK(k1());
      SX_CHECK(launch_vec<T>(ctx, n, MxJacobiUpdate{st, X, R[0], Z, P, Q, dinv}));
      return SX_OK;
    }
    for (int h2 = 0; h2 < 2; ++h2) {  // two iterations: r goes R0 -> R1 -> R0
      T* rin = R[h2];
      T* rout = R[h2 ^ 1];
      SX_CHECK(k1());
      if (!launch_pipe_gather<T, EpiMx2, GatherMxResid, true>(ctx, m->transpose->csr, nullptr, TW,
                                                               EpiMx2{ms, X, P, Q, rin, rout},
                                                               GatherMxResid{rin, Q, st}))
        return set_error(SX_ERR_CUDA, "CUDA error in the fused G^T step");
      if (!launch_pipe_gather<T, EpiMx3, GatherPlain<T>, true>(ctx, m->csr, TW, Z, EpiMx3{st, rout},
                                                                GatherPlain<T>{}))
        return set_error(SX_ERR_CUDA, "CUDA error in the fused G step");
    }
    return SX_OK;
  };
  const uint64_t key[8] = {4, (uint64_t)jac, a32->serial, m->serial, (uint64_t)n, (uint64_t)(uintptr_t)ws, 0, 0};
  double prev = rnorm;
  int stalls = 0;
  for (;;) {
    SX_CHECK(run_loop(ctx, ms, key, loop_as_graph(ctx, n), body));
    SX_CHECK(read_ctl(ctx, ms, &hs, sizeof(hs)));
    *inner += hs.cg.c.iterations;
    SX_CHECK(launch_vec<double>(ctx, n, IrFold{dx, X}));
    SX_CHECK(true_residual(h));
    rnorm = std::sqrt(h.rr);
    *rel = bnorm > 0 ? rnorm / bnorm : rnorm;
    *outer += 1;
    if (rnorm <= opt->tol * bnorm) { *converged = 1; break; }
    if (hs.cg.c.message == MSG_NOT_PD) break;
    if (*outer >= opt->max_outer) break;
    if (!(rnorm < 0.5 * prev)) {
      if (++stalls >= 2) break;
    } else {
      stalls = 0;
    }
    prev = rnorm;
    // replace the FP32 residual; p and q carry over (beta from the new r.z).
    // The captured body starts every pair of iterations from R[0], so the
    // replaced residual goes there whichever buffer the segment ended in.
    T* rcur = R[0];
    if (!jac && hs.rsel != 0) {
      hs.rsel = 0;
      SX_CHECK(write_bytes(ctx, &ms->rsel, &hs.rsel, sizeof(int)));
    }
    if (jac) {
      SX_CHECK(launch_vec<T>(ctx, n, MxStart{st, dr, rcur, Z, P, Q, dinv, true}));
    } else {
      SX_CHECK(launch_vec<double>(ctx, n, IrNarrow{dr, rcur, nullptr}));
      SX_CHECK(launch_apply<T>(ctx, m, rcur, Z, EpiPlain<T>{}));
      SX_CHECK(launch_vec<T>(ctx, n, MxStart{st, nullptr, rcur, Z, P, Q, nullptr, true}));
    }
  }
  return SX_OK;
}

int cg_mixed_replace(sx_ctx ctx, sx_op a64, sx_op a32, sx_op m, const double* db, double* dx, double* dr,
                     IrNorms* nrm, const sx_ir_options* opt, uint64_t* outer, uint64_t* inner,
                     double* rel, int* converged) {
  using T = float;
  const int64_t n = a64->nrows;
  if (!ctx->mx_unfused) {
    bool applied = false;
    SX_CHECK(cg_mixed_fused(ctx, a64, a32, m, db, dx, dr, nrm, opt, outer, inner, rel, converged, &applied));
    if (applied) {
      SX_CHECK(ic0_health(ctx, m));
      return SX_OK;
    }
  }
  SX_CHECK(check_prec(a32, m));
  const int pk = prec_kind(m);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * sizeof(T), 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 6, &ws, &dstate));
  // the layout of cg_run: the segment body is the same graph
  T* B = (T*)((char*)ws + 0 * vb);
  T* X = (T*)((char*)ws + 1 * vb);
  T* R = (T*)((char*)ws + 2 * vb);
  T* P = (T*)((char*)ws + 3 * vb);
  T* AP = (T*)((char*)ws + 4 * vb);
  T* Z = (T*)((char*)ws + 5 * vb);
  CgState<T>* st = (CgState<T>*)dstate;
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  const PrecFused<T> pf = prec_fused<T>(m);

  auto true_residual = [&](IrNorms& h) -> int {
    // FMA row sums: a few ulp per row, half the FP64 work
    SX_CHECK(launch_csr<double, EpiIrResid, true>(ctx, a64->csr, dx, dr, EpiIrResid{db, nrm}));
    SX_CHECK(read_ctl(ctx, nrm, &h, sizeof(h)));
    return SX_OK;
  };
  IrNorms h;
  SX_CHECK(true_residual(h));
  const double bnorm = std::sqrt(h.bb);
  double rnorm = std::sqrt(h.rr);
  *rel = bnorm > 0 ? rnorm / bnorm : rnorm;
  if (rnorm <= opt->tol * bnorm) {
    *converged = 1;
    return SX_OK;
  }
  const double delta = (opt->replace_factor > 0.0 && opt->replace_factor < 1.0) ? opt->replace_factor : 0.1;
  CgState<T> hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.c.max_iter = opt->max_inner;
  hs.rtol = (T)delta;                            // segment: ||r32|| drops by delta
  hs.atol = (T)(0.5 * opt->tol * bnorm);         // or reaches half the final target
  SX_CHECK(write_bytes(ctx, st, &hs, sizeof(hs)));
  SX_CHECK(launch_vec<double>(ctx, n, IrNarrow{dr, R, B}));
  if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * sizeof(T), ctx->stream));
  if (pk == PK_GENERAL) SX_CHECK(launch_apply<T>(ctx, m, R, Z, EpiPlain<T>{}));
  SX_CHECK(launch_vec<T>(ctx, n, CgSetup<T>{st, B, R, Z, P, pf}));
  auto body = [&]() -> int {
    SX_CHECK(launch_apply<T>(ctx, a32, P, AP, EpiCgPap<T>{st, P}));
    SX_CHECK(launch_vec<T>(ctx, n, CgUpdate<T>{st, X, R, P, AP, pf}));
    if (pk == PK_GENERAL) {
      SX_CHECK(launch_apply<T>(ctx, m, R, Z, EpiCgRz<T>{st, R}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, CgP<T>{st, P, R, Z, pf}));
    return SX_OK;
  };
  const uint64_t key[8] = {1, (uint64_t)sizeof(T), a32->serial, m ? m->serial : 0,
                           (uint64_t)n, (uint64_t)(uintptr_t)ws, (uint64_t)pk, 0};
  double prev = rnorm;
  int stalls = 0;
  for (;;) {
    SX_CHECK(run_loop(ctx, st, key, op_graphable(a32) && op_graphable(m), body));
    SX_CHECK(read_ctl(ctx, st, &hs, sizeof(hs)));
    *inner += hs.c.iterations;
    SX_CHECK(launch_vec<double>(ctx, n, IrFold{dx, X}));
    SX_CHECK(true_residual(h));
    rnorm = std::sqrt(h.rr);
    *rel = bnorm > 0 ? rnorm / bnorm : rnorm;
    *outer += 1;
    if (rnorm <= opt->tol * bnorm) { *converged = 1; break; }
    if (hs.c.message == MSG_NOT_PD) break;  // FP32 p.Ap <= 0: no further progress in FP32
    if (*outer >= opt->max_outer) break;
    if (!(rnorm < 0.5 * prev)) {
      if (++stalls >= 2) break;  // FP32 iteration has stagnated
    } else {
      stalls = 0;
    }
    prev = rnorm;
    if (pk == PK_GENERAL) {
      SX_CHECK(launch_vec<double>(ctx, n, IrNarrow{dr, R, nullptr}));
      SX_CHECK(launch_apply<T>(ctx, m, R, Z, EpiPlain<T>{}));
      SX_CHECK(launch_vec<T>(ctx, n, IrRz{st, R, Z}));
    } else {
      SX_CHECK(launch_vec<T>(ctx, n, IrNarrowRz{st, dr, R, pf}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, IrP{st, P, R, Z, pf}));
  }
  SX_CHECK(ic0_health(ctx, m));
  return SX_OK;
}

// =============================================================== BiCGSTAB
template <typename T>
struct BiState {
  LoopCtl c;
  T rho, rho_old, alpha, omega, beta, rnorm, tol, rtol, atol, result_norm;
  int x_is_y, pad2;
};

// r_hat = r, v = p = 0, ||r||, ||b||, initial exits, first rho
// (iterative.rs:416-447, 450-465)
template <typename T>
struct BiSetup {
  BiState<T>* st;
  const T *b, *r;
  T *rhat, *v, *p;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    T ri = r[i];
    rhat[i] = ri;
    v[i] = T(0);
    p[i] = T(0);
    a.a += ri * ri;
    a.b += b[i] * b[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    T rnorm = sqrt(t.a);
    T bnorm = sqrt(t.b);
    st->rnorm = rnorm;
    st->result_norm = rnorm;
    st->tol = fmax(st->atol, st->rtol * bnorm);
    if (rnorm <= st->tol) {
      st->c.status = ST_DONE;
      st->c.converged = 1;
      st->c.message = MSG_CONVERGED_INITIAL;
      return;
    }
    st->rho_old = T(1);
    st->alpha = T(0);
    st->omega = T(1);
    if (st->c.max_iter == 0) {
      st->c.status = ST_DONE;
      st->c.message = MSG_MAX_ITER;
      return;
    }
    // rho = (r_hat, r) with r_hat == r: the same products as ||r||^2
    T rho = t.a;
    st->rho = rho;
    if (fabs(rho) < eps_of<T>() * T(10)) {
      st->c.status = ST_DONE;
      st->c.message = MSG_BD_RHO;
      return;
    }
    st->beta = (rho / st->rho_old) * (st->alpha / st->omega);
  }
};

// p = r + beta (p - omega v); p~ = M1 p for fused M1 (iterative.rs:467-475)
template <typename T>
struct BiP {
  BiState<T>* st;
  T *p, *pt;
  const T *r, *v;
  PrecFused<T> pf1;
  int store_pt;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    T pi = add_rn(r[i], mul_rn(st->beta, sub_rn(p[i], mul_rn(st->omega, v[i]))));
    p[i] = pi;
    if (store_pt) pt[i] = pf1.apply(i, pi);
  }
  __device__ void finish(const Acc3<T>&) const {}
};

// (r_hat, v), alpha and its exits (iterative.rs:486-507)
template <typename T>
struct EpiBiRhoV {
  BiState<T>* st;
  const T* rhat;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t i, T y, Acc3<T>& a) const { a.a += rhat[i] * y; }
  __device__ void finish(const Acc3<T>& t) const {
    T den = t.a;
    if (fabs(den) < eps_of<T>() * T(10)) {
      st->c.status = ST_DONE;
      st->c.message = MSG_BD_RHAT_V;
      st->result_norm = st->rnorm;
      return;
    }
    T alpha = st->rho / den;
    st->alpha = alpha;
    if (!isfinite(alpha)) {
      st->c.status = ST_DONE;
      st->c.message = MSG_BD_ALPHA;
      st->result_norm = st->rnorm;
    }
  }
};

// y = x + alpha p~; s = r - alpha v; ||s|| (iterative.rs:510-533)
template <typename T>
struct BiS {
  BiState<T>* st;
  const T *x, *pt, *r, *v;
  T *y, *s, *stl;
  PrecFused<T> pf1;
  int store_st;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T alpha = st->alpha;
    y[i] = add_rn(x[i], mul_rn(alpha, pt[i]));
    T si = sub_rn(r[i], mul_rn(alpha, v[i]));
    s[i] = si;
    if (store_st) stl[i] = pf1.apply(i, si);
    a.a += si * si;
  }
  __device__ void finish(const Acc3<T>& t) const {
    T snorm = sqrt(t.a);
    if (snorm <= st->tol) {
      st->c.status = ST_DONE;
      st->c.converged = 1;
      st->c.message = MSG_CONVERGED;
      st->c.iterations += 1;
      st->result_norm = snorm;
      st->x_is_y = 1;
    }
  }
};

// (t, s), (t, t), omega and its exits (iterative.rs:550-574)
template <typename T>
struct EpiBiT {
  BiState<T>* st;
  const T* s;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t i, T t, Acc3<T>& a) const {
    a.a += t * s[i];
    a.b += t * t;
  }
  __device__ void finish(const Acc3<T>& tot) const {
    const T e10 = eps_of<T>() * T(10);
    T ts = tot.a, tt = tot.b;
    if (tt < e10) {
      st->c.status = ST_DONE;
      st->c.message = MSG_BD_TT;
      st->result_norm = st->rnorm;
      return;
    }
    T omega = ts / tt;
    st->omega = omega;
    if (!isfinite(omega) || fabs(omega) < e10) {
      st->c.status = ST_DONE;
      st->c.message = MSG_BD_OMEGA;
      st->result_norm = st->rnorm;
    }
  }
};

// x = y + omega s~ (then M2 x); r = s - omega t; ||r||; next rho and the
// loop bookkeeping (iterative.rs:577-606, 450-465).  mode 0: whole step;
// mode 1: updates only (x into xt for a general M2); mode 2: reductions only.
template <typename T>
struct BiR {
  BiState<T>* st;
  T *x, *r;
  const T *y, *stl, *s, *t, *rhat;
  T* xt;
  PrecFused<T> pf2;
  int mode;
  static constexpr bool kReduce = true;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (mode != 1 && blockIdx.x == 0 && threadIdx.x == 0)
        set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    if (mode != 2) {
      const T omega = st->omega;
      T xi = add_rn(y[i], mul_rn(omega, stl[i]));
      if (mode == 1) xt[i] = xi;
      else x[i] = pf2.apply(i, xi);
      r[i] = sub_rn(s[i], mul_rn(omega, t[i]));
    }
    if (mode != 1) {
      T ri = r[i];
      a.a += ri * ri;
      a.b += rhat[i] * ri;
    }
  }
  __device__ void finish(const Acc3<T>& tot) const {
    if (mode == 1) return;
    T rnorm = sqrt(tot.a);
    st->rnorm = rnorm;
    st->result_norm = rnorm;
    if (rnorm <= st->tol) {
      st->c.status = ST_DONE;
      st->c.converged = 1;
      st->c.message = MSG_CONVERGED;
      st->c.iterations += 1;
    } else {
      st->rho_old = st->rho;
      st->c.iterations += 1;
      if (st->c.iterations >= st->c.max_iter) {
        st->c.status = ST_DONE;
        st->c.message = MSG_MAX_ITER;
      } else {
        T rho = tot.b;
        st->rho = rho;
        if (fabs(rho) < eps_of<T>() * T(10)) {
          st->c.status = ST_DONE;
          st->c.message = MSG_BD_RHO;
        } else {
          st->beta = (rho / st->rho_old) * (st->alpha / st->omega);
        }
      }
    }
    if (st->c.budget > 0) st->c.budget -= 1;
    set_cond(st->c.use_cond, st->c.cond,
             (st->c.status == ST_RUNNING && st->c.budget > 0) ? 1u : 0u);
  }
};

template <typename T>
static int bicgstab_run(sx_ctx ctx, sx_op a, const void* b, const sx_bicgstab_options* opt,
                        void* x_out, sx_mem mem, sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m1 = opt->left_preconditioner, m2 = opt->right_preconditioner;
  SX_CHECK(check_prec(a, m1));
  SX_CHECK(check_prec(a, m2));
  const int k1 = prec_kind(m1), k2 = prec_kind(m2);
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 13, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R = V(2), *RH = V(3), *P = V(4), *PT = V(5), *VV = V(6), *Y = V(7),
    *S = V(8), *STL = V(9), *TT = V(10), *TMP = V(11), *XT = V(12);
  BiState<T>* st = (BiState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  BiState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  const PrecFused<T> pf1 = prec_fused<T>(m1), pf2 = prec_fused<T>(m2);
  SX_CHECK(launch_apply<T>(ctx, a, X, R, EpiResid<T>{B}));
  SX_CHECK(launch_vec<T>(ctx, n, BiSetup<T>{st, B, R, RH, VV, P}));
  // p~ and s~: the same buffer as p / s when there is no M1
  T* ptil = (k1 == PK_NONE) ? P : PT;
  T* stil = (k1 == PK_NONE) ? S : STL;
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, BiP<T>{st, P, PT, R, VV, pf1, (k1 == PK_DIAG || k1 == PK_SCALED) ? 1 : 0}));
    if (k1 == PK_GENERAL) SX_CHECK(launch_apply<T>(ctx, m1, P, PT, EpiSkip<T, BiState<T>>{st}));
    if (!m2) {
      SX_CHECK(launch_apply<T>(ctx, a, ptil, VV, EpiBiRhoV<T>{st, RH}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, ptil, TMP, EpiSkip<T, BiState<T>>{st}));
      SX_CHECK(launch_apply<T>(ctx, m2, TMP, VV, EpiBiRhoV<T>{st, RH}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, BiS<T>{st, X, ptil, R, VV, Y, S, STL, pf1,
                                          (k1 == PK_DIAG || k1 == PK_SCALED) ? 1 : 0}));
    if (k1 == PK_GENERAL) SX_CHECK(launch_apply<T>(ctx, m1, S, STL, EpiSkip<T, BiState<T>>{st}));
    if (!m2) {
      SX_CHECK(launch_apply<T>(ctx, a, stil, TT, EpiBiT<T>{st, S}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, stil, TMP, EpiSkip<T, BiState<T>>{st}));
      SX_CHECK(launch_apply<T>(ctx, m2, TMP, TT, EpiBiT<T>{st, S}));
    }
    if (k2 == PK_GENERAL) {
      SX_CHECK(launch_vec<T>(ctx, n, BiR<T>{st, X, R, Y, stil, S, TT, RH, XT, pf2, 1}));
      SX_CHECK(launch_apply<T>(ctx, m2, XT, X, EpiSkip<T, BiState<T>>{st}));
      SX_CHECK(launch_vec<T>(ctx, n, BiR<T>{st, X, R, Y, stil, S, TT, RH, XT, pf2, 2}));
    } else {
      SX_CHECK(launch_vec<T>(ctx, n, BiR<T>{st, X, R, Y, stil, S, TT, RH, XT, pf2, 0}));
    }
    return SX_OK;
  };
  const uint64_t key[8] = {2, (uint64_t)sizeof(T), a->serial, m1 ? m1->serial : 0,
                           m2 ? m2->serial : 0, (uint64_t)n, (uint64_t)(uintptr_t)ws, 0};
  SX_CHECK(run_loop(ctx, st, key,
                    op_graphable(a) && op_graphable(m1) && op_graphable(m2), body));
  SX_CHECK(ic0_health(ctx, m1));
  SX_CHECK(ic0_health(ctx, m2));
  SX_CHECK(read_ctl(ctx, st, &h, sizeof(h)));
  if (h.x_is_y) {
    // x = y, then x = M2 x (iterative.rs:519-524)
    if (m2) SX_CHECK(launch_apply<T>(ctx, m2, Y, X, EpiPlain<T>{}));
    else if (n > 0) SX_CUDA(cudaMemcpyAsync(X, Y, n * w, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  SX_CHECK(vec_out(ctx, x_out, X, n * w, mem));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (res) {
    res->iterations = h.c.iterations;
    res->residual_norm = (double)h.result_norm;
    res->converged = h.c.converged;
    res->message = h.c.message;
  }
  return SX_OK;
}

// ================================================================== GMRES
// One WHILE iteration = one restart cycle (iterative.rs:695-803).  Arnoldi
// step j is captured as: w = M A v_j; for i = 0..j one fused kernel that
// finishes the previous projection (w -= h_{i-1,j} v_{i-1}) and forms
// h_ij = (v_i, w) -- modified Gram-Schmidt in the reference's order; a final
// kernel subtracts the last projection and forms ||w||, whose finishing
// block also applies the Givens rotations; then v_{j+1} = w / ||w||.
// Kernels of step j return at once unless the cycle is still at step j.
template <typename T>
struct GmState {
  LoopCtl c;
  T rnorm, tol, rtol, atol, hnorm;
  int restart, j, active;  // j: inner_iter of the current cycle; active: cycle running
  int stalled;             // a cycle ended with j = 0: the next would repeat it
  unsigned long long outer;
};

template <typename T>
struct GmArrays {
  T* h;   // (restart+1) x restart, row-major h[i*restart + j]
  T* cs;  // restart
  T* sn;  // restart
  T* s;   // restart + 1
  T* y;   // restart
};

// ||r|| and the setup of a cycle: v_0 = r / ||r||, s = [||r||, 0, ...]
template <typename T>
struct GmStart {
  GmState<T>* st;
  GmArrays<T> g;
  const T* r;
  T* v0;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    // iterative.rs:704: v[0] = r / rnorm
    v0[i] = r[i] / st->rnorm;
  }
  __device__ void finish(const Acc3<T>&) const {
    const int R = st->restart;
    for (int q = 0; q < (R + 1) * R; ++q) g.h[q] = T(0);
    for (int q = 0; q < R; ++q) { g.cs[q] = T(0); g.sn[q] = T(0); }
    for (int q = 0; q <= R; ++q) g.s[q] = T(0);
    g.s[0] = st->rnorm;
    st->j = 0;
    st->active = (R > 0 && st->outer < st->c.max_iter) ? 1 : 0;
  }
};

// w = A v_j (then M w) while the cycle is at step jj
template <typename T>
struct EpiGmW {
  GmState<T>* st;
  int jj;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != jj; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// MGS projection i of step jj: w -= h_{i-1,jj} v_{i-1} (i > 0); h_{i,jj} = (v_i, w)
template <typename T>
struct GmMgs {
  GmState<T>* st;
  GmArrays<T> g;
  T* w;
  const T *vprev, *vi;
  int i, jj;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != jj; }
  __device__ void elem(int64_t k, Acc3<T>& a) const {
    T wk = w[k];
    if (i > 0) {
      wk = sub_rn(wk, mul_rn(g.h[(i - 1) * st->restart + jj], vprev[k]));
      w[k] = wk;
    }
    a.a += vi[k] * wk;
  }
  __device__ void finish(const Acc3<T>& t) const { g.h[i * st->restart + jj] = t.a; }
};

// last projection, ||w||, breakdown, Givens rotations, convergence
// (iterative.rs:719-768)
template <typename T>
struct GmNorm {
  GmState<T>* st;
  GmArrays<T> g;
  T* w;
  const T* vj;
  int jj;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != jj; }
  __device__ void elem(int64_t k, Acc3<T>& a) const {
    T wk = sub_rn(w[k], mul_rn(g.h[jj * st->restart + jj], vj[k]));
    w[k] = wk;
    a.a += wk * wk;
  }
  __device__ void finish(const Acc3<T>& t) const {
    const int R = st->restart;
    T* h = g.h;
    const int j = jj;
    T hn = sqrt(t.a);
    h[(j + 1) * R + j] = hn;
    st->hnorm = hn;
    if (hn < eps_of<T>() * T(10)) {
      st->active = 0;  // happy breakdown: column j is dropped
      return;
    }
    for (int i = 0; i < j; ++i) {
      T a = h[i * R + j], b = h[(i + 1) * R + j];
      T temp = add_rn(mul_rn(g.cs[i], a), mul_rn(g.sn[i], b));
      h[(i + 1) * R + j] = add_rn(mul_rn(-g.sn[i], a), mul_rn(g.cs[i], b));
      h[i * R + j] = temp;
    }
    T hjj = h[j * R + j], hj1 = h[(j + 1) * R + j];
    T rho = sqrt(add_rn(mul_rn(hjj, hjj), mul_rn(hj1, hj1)));
    g.cs[j] = hjj / rho;
    g.sn[j] = hj1 / rho;
    h[j * R + j] = rho;
    h[(j + 1) * R + j] = T(0);
    T temp = add_rn(mul_rn(g.cs[j], g.s[j]), mul_rn(g.sn[j], g.s[j + 1]));
    g.s[j + 1] = add_rn(mul_rn(-g.sn[j], g.s[j]), mul_rn(g.cs[j], g.s[j + 1]));
    g.s[j] = temp;
    st->j = j + 1;
    // v_{j+1} is normalised by the next kernel with st->hnorm
    st->active = 2;  // normalise pending, then continue
  }
};

// v_{j+1} = w / h_{j+1,j}; decide whether the cycle continues
template <typename T>
struct GmNormalize {
  GmState<T>* st;
  GmArrays<T> g;
  const T* w;
  T* vnext;
  int jj;
  static constexpr bool kReduce = true;
  __device__ bool skip() const {
    return st->c.status != ST_RUNNING || st->active != 2 || st->j != jj + 1;
  }
  __device__ void elem(int64_t k, Acc3<T>&) const { vnext[k] = w[k] / st->hnorm; }
  __device__ void finish(const Acc3<T>&) const {
    const int j = st->j;
    bool more = j < st->restart && (unsigned long long)j + st->outer < st->c.max_iter;
    if (fabs(g.s[j]) <= st->tol) more = false;
    st->active = more ? 1 : 0;
  }
};

// back substitution (iterative.rs:771-779), one thread
template <typename T>
__global__ void k_gm_backsub(GmState<T>* st, GmArrays<T> g) {
  if (st->c.status != ST_RUNNING) return;
  const int R = st->restart, j = st->j;
  for (int i = j - 1; i >= 0; --i) {
    T yi = g.s[i];
    for (int q = i + 1; q < j; ++q) yi = sub_rn(yi, mul_rn(g.h[i * R + q], g.y[q]));
    g.y[i] = yi / g.h[i * R + i];
  }
}

// x += sum_i y_i v_i in the reference's order (iterative.rs:782-786)
template <typename T>
struct GmX {
  GmState<T>* st;
  GmArrays<T> g;
  T* x;
  const T* vbase;
  size_t vstride;  // elements between basis vectors
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t k, Acc3<T>&) const {
    const int j = st->j;
    T xk = x[k];
    for (int i = 0; i < j; ++i) xk = add_rn(xk, mul_rn(g.y[i], vbase[(size_t)i * vstride + k]));
    x[k] = xk;
  }
  __device__ void finish(const Acc3<T>&) const {}
};

// ||r|| after a cycle, outer count, loop condition (iterative.rs:789-803)
template <typename T>
struct GmEnd {
  GmState<T>* st;
  const T* r;
  static constexpr bool kReduce = true;
  __device__ bool skip() const {
    if (st->c.status != ST_RUNNING) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(st->c.use_cond, st->c.cond, 0u);
      return true;
    }
    return false;
  }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += r[i] * r[i]; }
  __device__ void finish(const Acc3<T>& t) const {
    T rnorm = sqrt(t.a);
    st->rnorm = rnorm;
    st->outer += (unsigned long long)st->j;
    st->c.iterations = st->outer;
    if (rnorm <= st->tol || !(st->outer < st->c.max_iter)) {
      st->c.status = ST_DONE;
      st->c.converged = rnorm <= st->tol ? 1 : 0;
      st->c.message = st->c.converged ? MSG_CONVERGED : MSG_MAX_ITER;
    } else if (st->j == 0) {
      // a breakdown at the first Arnoldi step (A r0 parallel to r0) left x,
      // r and the count unchanged: the reference's loop would repeat this
      // cycle forever (iterative.rs:697-808)
      st->c.status = ST_DONE;
      st->stalled = 1;
    }
    if (st->c.budget > 0) st->c.budget -= 1;
    set_cond(st->c.use_cond, st->c.cond,
             (st->c.status == ST_RUNNING && st->c.budget > 0) ? 1u : 0u);
  }
};

// initial ||r|| (after the optional M r) and ||b||
template <typename T>
struct GmInit {
  GmState<T>* st;
  const T *r, *b;
  static constexpr bool kReduce = true;
  static constexpr bool kVec4 = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    a.a += r[i] * r[i];
    a.b += b[i] * b[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rnorm = sqrt(t.a);
    st->tol = fmax(st->atol, st->rtol * sqrt(t.b));
    st->outer = 0;
    if (!(0 < st->c.max_iter && st->rnorm > st->tol)) {
      st->c.status = ST_DONE;
      st->c.converged = st->rnorm <= st->tol ? 1 : 0;
      st->c.message = st->c.converged ? MSG_CONVERGED : MSG_MAX_ITER;
    }
  }
};

template <typename T>
static int gmres_run(sx_ctx ctx, sx_op a, const void* b, const sx_gmres_options* opt, void* x_out,
                     sx_mem mem, sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m = opt->preconditioner;
  SX_CHECK(check_prec(a, m));
  const uint64_t restart64 = std::min<uint64_t>(opt->restart, (uint64_t)n);
  if (restart64 > 4096)
    return set_error(SX_ERR_VALUE, "Value error: restart above 4096 is not supported on the device");
  const int R = (int)restart64;
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  const size_t small = align_up((size_t)((R + 1) * (R + 1) * 2 + 4 * (R + 2)) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * (6 + (size_t)R + 1) + small, &ws, &dstate));
  auto V = [&](size_t i) { return (T*)((char*)ws + i * vb); };
  T *B = V(0), *X = V(1), *Rv = V(2), *W = V(3), *TMP = V(4), *AX = V(5);
  T* basis = V(6);  // R + 1 vectors, stride vb / w elements
  const size_t vstride = vb / w;
  T* sm = (T*)((char*)ws + vb * (6 + (size_t)R + 1));
  GmArrays<T> g;
  g.h = sm;
  g.cs = g.h + (size_t)(R + 1) * std::max(R, 1);
  g.sn = g.cs + std::max(R, 1);
  g.s = g.sn + std::max(R, 1);
  g.y = g.s + R + 1;
  (void)AX;
  GmState<T>* st = (GmState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  GmState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  h.restart = R;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  // r = M (b - A x); ||r||; ||b|| (iterative.rs:677-690)
  if (m) {
    SX_CHECK(launch_apply<T>(ctx, a, X, TMP, EpiResid<T>{B}));
    SX_CHECK(launch_apply<T>(ctx, m, TMP, Rv, EpiPlain<T>{}));
  } else {
    SX_CHECK(launch_apply<T>(ctx, a, X, Rv, EpiResid<T>{B}));
  }
  SX_CHECK(launch_vec<T>(ctx, n, GmInit<T>{st, Rv, B}));
  {
    GmState<T> hs;
    SX_CHECK(read_ctl(ctx, st, &hs, sizeof(hs)));
    if (hs.c.status == ST_RUNNING && R == 0)
      return set_error(SX_ERR_VALUE,
                       "Value error: restart = 0 makes no progress (the reference loops forever)");
  }
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, GmStart<T>{st, g, Rv, basis}));
    for (int j = 0; j < R; ++j) {
      T* vj = basis + (size_t)j * vstride;
      if (m) {
        SX_CHECK(launch_apply<T>(ctx, a, vj, TMP, EpiGmW<T>{st, j}));
        SX_CHECK(launch_apply<T>(ctx, m, TMP, W, EpiGmW<T>{st, j}));
      } else {
        SX_CHECK(launch_apply<T>(ctx, a, vj, W, EpiGmW<T>{st, j}));
      }
      for (int i = 0; i <= j; ++i) {
        const T* vprev = i > 0 ? basis + (size_t)(i - 1) * vstride : nullptr;
        SX_CHECK(launch_vec<T>(ctx, n, GmMgs<T>{st, g, W, vprev, basis + (size_t)i * vstride, i, j}));
      }
      SX_CHECK(launch_vec<T>(ctx, n, GmNorm<T>{st, g, W, vj, j}));
      SX_CHECK(launch_vec<T>(ctx, n, GmNormalize<T>{st, g, W, basis + (size_t)(j + 1) * vstride, j}));
    }
    k_gm_backsub<T><<<1, 1, 0, ctx->stream>>>(st, g);
    ctx->launches++;
    SX_CHECK(launch_vec<T>(ctx, n, GmX<T>{st, g, X, basis, vstride}));
    if (m) {
      SX_CHECK(launch_apply<T>(ctx, a, X, TMP, EpiResid<T>{B}));
      SX_CHECK(launch_apply<T>(ctx, m, TMP, Rv, EpiPlain<T>{}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, X, Rv, EpiResid<T>{B}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, GmEnd<T>{st, Rv}));
    return SX_OK;
  };
  const uint64_t key[8] = {3, (uint64_t)sizeof(T), a->serial, m ? m->serial : 0,
                           (uint64_t)n, (uint64_t)(uintptr_t)ws, (uint64_t)R, 0};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m), body));
  SX_CHECK(ic0_health(ctx, m));
  SX_CHECK(read_ctl(ctx, st, &h, sizeof(h)));
  if (h.stalled)
    return set_error(SX_ERR_COMPUTATION,
                     "Computation error: gmres cannot advance: breakdown at the first Arnoldi step "
                     "(the reference loops forever)");
  SX_CHECK(vec_out(ctx, x_out, X, n * w, mem));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (res) {
    res->iterations = h.outer;
    res->residual_norm = (double)h.rnorm;
    res->converged = h.rnorm <= h.tol ? 1 : 0;
    res->message = res->converged ? MSG_CONVERGED : MSG_MAX_ITER;
  }
  return SX_OK;
}

}  // namespace sx

using namespace sx;

extern "C" {

void sx_cg_options_default(sx_cg_options* o) {
  o->max_iter = 1000;
  o->rtol = 1e-8;
  o->atol = 1e-12;
  o->x0 = nullptr;
  o->preconditioner = nullptr;
}
void sx_bicgstab_options_default(sx_bicgstab_options* o) {
  o->max_iter = 1000;
  o->rtol = 1e-8;
  o->atol = 1e-12;
  o->x0 = nullptr;
  o->left_preconditioner = nullptr;
  o->right_preconditioner = nullptr;
}
void sx_gmres_options_default(sx_gmres_options* o) {
  o->max_iter = 1000;
  o->restart = 30;
  o->rtol = 1e-8;
  o->atol = 1e-12;
  o->x0 = nullptr;
  o->preconditioner = nullptr;
}

int sx_ctx_set_cg_recurrence(sx_ctx ctx, int on) {
  if (!ctx) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx");
  ctx->cg_recurrence = on != 0;
  return clear_error();
}

int sx_cg(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_cg_options* opt,
          void* x_out, sx_mem mem, sx_iter_result* res) {
  SX_CHECK(solver_checks(ctx, a, b, b_len, x_out, "CG"));
  sx_cg_options d;
  if (!opt) { sx_cg_options_default(&d); opt = &d; }
  int rc = a->dtype == SX_F64 ? cg_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : cg_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_bicgstab(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicgstab_options* opt,
                void* x_out, sx_mem mem, sx_iter_result* res) {
  SX_CHECK(solver_checks(ctx, a, b, b_len, x_out, "BiCGSTAB"));
  sx_bicgstab_options d;
  if (!opt) { sx_bicgstab_options_default(&d); opt = &d; }
  int rc = a->dtype == SX_F64 ? bicgstab_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : bicgstab_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_gmres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_gmres_options* opt,
             void* x_out, sx_mem mem, sx_iter_result* res) {
  SX_CHECK(solver_checks(ctx, a, b, b_len, x_out, "GMRES"));
  sx_gmres_options d;
  if (!opt) { sx_gmres_options_default(&d); opt = &d; }
  int rc = a->dtype == SX_F64 ? gmres_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : gmres_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

void sx_solver_cache_release(sx_ctx ctx) {
  if (!ctx || !ctx->solver_cache) return;
  SolverCache* c = (SolverCache*)ctx->solver_cache;
  drop_graphs(c);
  dev_free(c->ws);
  dev_free(c->state);
  delete c;
  ctx->solver_cache = nullptr;
}

}  // extern "C"
