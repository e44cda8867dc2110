// More Krylov solvers of scirs2-sparse on the device: bicg
// (linalg/iterative.rs:189-345), cgs (linalg/cgs.rs:15-193), qmr
// (linalg/qmr.rs:44-259), minres (linalg/minres.rs:66-257) and lgmres
// (linalg/lgmres.rs:58-327).
//
// Same execution model as cg / bicgstab / gmres: every scalar of the
// recurrence lives in a device-side state block, the reductions are fused
// into the kernels that produce their operands, the last block of each
// reduction takes the reference's scalar step and its exits in the
// reference's order, and one iteration (for lgmres: one outer cycle) is
// captured into the body of a CUDA-graph WHILE loop.  Kernels of an ended
// solve return at once.  Vector updates round every product and sum
// separately, as the reference's loops do; dot products are tree sums.
// Operators and preconditioners go through launch_apply, so every operator
// kind works in every slot; the adjoint needed by bicg and qmr is the
// cached transpose of a CSR matrix or the operator itself for the
// self-adjoint kinds.

#include <charconv>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>

#include "sx_solver.cuh"

namespace sx {
namespace {

// A^H as an operator (LinearOperator::rmatvec).  CSR: the cached transpose
// (interface.rs:281-285 transposes on every call; same arrays); sums and
// products: composites of the operands' adjoints (interface.rs:332-345,
// :382-395), kept on the handle; the preconditioners and elementwise
// operators are their own adjoints; a host operator has none
// (interface.rs:40-45).
int adjoint_op(sx_ctx ctx, sx_op op, sx_op* out) {
  *out = nullptr;
  if (!op) return SX_OK;
  switch (op->kind) {
    case SX_OP_CSR:
      SX_CHECK(ensure_transpose(ctx, op));
      *out = op->transpose;
      return SX_OK;
    case SX_OP_HOST:
    case SX_OP_ILU0:  // preconditioners.rs:189-191, :378-380
    case SX_OP_SSOR:
      return set_error(SX_ERR_OPERATION_NOT_SUPPORTED,
                       "Operation not supported: adjoint not implemented for this operator");
    case SX_OP_ZERO:
      if (!op->transpose)
        SX_CHECK(sx_op_zero(ctx, (sx_dtype)op->dtype, (uint64_t)op->ncols, (uint64_t)op->nrows, &op->transpose));
      *out = op->transpose;
      return SX_OK;
    case SX_OP_SUM:
    case SX_OP_PRODUCT: {
      if (!op->transpose) {
        int la = 0, lb = 0;
        sx_op_has_adjoint(op->left, &la);
        sx_op_has_adjoint(op->right, &lb);
        if (!la || !lb)
          return set_error(SX_ERR_OPERATION_NOT_SUPPORTED,
                           "Operation not supported: adjoint not supported for one or both operators");
        sx_op l = nullptr, r = nullptr;
        SX_CHECK(adjoint_op(ctx, op->left, &l));
        SX_CHECK(adjoint_op(ctx, op->right, &r));
        if (op->kind == SX_OP_SUM) SX_CHECK(sx_op_sum(ctx, l, r, &op->transpose));
        else SX_CHECK(sx_op_product(ctx, r, l, &op->transpose));
      }
      *out = op->transpose;
      return SX_OK;
    }
    default:
      *out = op;
      return SX_OK;
  }
}

// y = M x when M is set, else nothing (the caller aliases y to x)
template <typename T, class S>
int apply_opt(sx_ctx ctx, sx_op m, const T* x, T* y, const S* st) {
  if (!m) return SX_OK;
  return launch_apply<T>(ctx, m, x, y, EpiSkip<T, S>{st});
}

template <typename T>
__device__ __forceinline__ T eps10() { return eps_of<T>() * T(10); }

// The last kernel of an iteration re-arms the WHILE condition; once the
// solve has ended it clears it.
__device__ __forceinline__ void loop_tail(LoopCtl& c) {
  if (c.budget > 0) c.budget -= 1;
  set_cond(c.use_cond, c.cond, (c.status == ST_RUNNING && c.budget > 0) ? 1u : 0u);
}
__device__ __forceinline__ bool ended_tail(const LoopCtl& c) {
  if (c.status != ST_RUNNING) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(c.use_cond, c.cond, 0u);
    return true;
  }
  return false;
}
__device__ __forceinline__ void finish_loop(LoopCtl& c, int msg, int converged) {
  c.status = ST_DONE;
  c.message = msg;
  c.converged = converged;
}

// Reduction epilogue of an operator apply: a.a += u[i] y_i, a.b += y_i^2,
// a.c += w[i] y_i (w optional); the state's step() takes the totals.
template <typename T, class S, int STEP>
struct EpiDots {
  S* st;
  const T *u, *w;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t i, T y, Acc3<T>& a) const {
    if (u) a.a += u[i] * y;
    a.b += y * y;
    if (w) a.c += w[i] * y;
  }
  __device__ void finish(const Acc3<T>& t) const { st->template step<STEP>(t); }
};

// b - A x, skipped once the solve has ended
template <typename T, class S>
struct EpiResidSkip {
  const S* st;
  const T* b;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t i, T ax) const { return sub_rn(b[i], ax); }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// ===================================================================== BiCG
template <typename T>
struct BgState {
  LoopCtl c;
  T rho_old, rho, alpha, beta, rnorm, tol, rtol, atol, result_norm;
  // den = (p*, q), alpha (iterative.rs:267-280)
  template <int K>
  __device__ void step(const Acc3<T>& t) {
    if constexpr (K == 0) {
      const T den = t.a;
      if (fabs(den) < eps10<T>()) {
        result_norm = rnorm;
        finish_loop(c, MSG_BICG_PQ, 0);
        return;
      }
      alpha = rho_old / den;
    } else {
      // rho = (r*, z), beta (iterative.rs:313-328)
      const T r = t.a;
      if (fabs(r) < eps10<T>()) {
        c.iterations += 1;
        result_norm = rnorm;
        finish_loop(c, MSG_BICG_RHO, 0);
        return;
      }
      rho = r;
      beta = r / rho_old;
    }
  }
};

// p = z, p* = z*, rho_old = (r*, z), ||b||, ||r|| (iterative.rs:231-253)
template <typename T>
struct BgSetup {
  BgState<T>* st;
  const T *b, *r, *rs, *z, *zs;
  T *p, *ps;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    p[i] = z[i];
    ps[i] = zs[i];
    a.a += rs[i] * z[i];
    a.b += b[i] * b[i];
    a.c += r[i] * r[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rho_old = t.a;
    st->tol = fmax(st->atol, mul_rn(st->rtol, sqrt(t.b)));
    st->rnorm = sqrt(t.c);
    st->result_norm = st->rnorm;
    if (st->c.max_iter == 0) finish_loop(st->c, MSG_MAX_ITER, 0);
  }
};

// x += alpha p, r -= alpha q, r* -= alpha q*, ||r|| and its exit; without
// preconditioners also rho = (r*, r) (iterative.rs:283-311)
template <typename T>
struct BgUpdate {
  BgState<T>* st;
  T *x, *r, *rs;
  const T *p, *q, *qs;
  int fuse_rho;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T al = st->alpha;
    x[i] = add_rn(x[i], mul_rn(al, p[i]));
    const T ri = sub_rn(r[i], mul_rn(al, q[i]));
    const T rsi = sub_rn(rs[i], mul_rn(al, qs[i]));
    r[i] = ri;
    rs[i] = rsi;
    a.a += ri * ri;
    a.b += rsi * ri;
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rnorm = sqrt(t.a);
    st->result_norm = st->rnorm;
    if (st->rnorm <= st->tol) {
      st->c.iterations += 1;
      finish_loop(st->c, MSG_CONVERGED, 1);
      return;
    }
    if (fuse_rho) st->template step<1>(Acc3<T>{t.b, T(0), T(0)});
  }
};

template <typename T>
struct BgRho {
  BgState<T>* st;
  const T *rs, *z;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += rs[i] * z[i]; }
  __device__ void finish(const Acc3<T>& t) const { st->template step<1>(t); }
};

// p = z + beta p, p* = z* + beta p*; loop bookkeeping (iterative.rs:331-342)
template <typename T>
struct BgP {
  BgState<T>* st;
  T *p, *ps;
  const T *z, *zs;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return ended_tail(st->c); }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    const T b = st->beta;
    p[i] = add_rn(z[i], mul_rn(b, p[i]));
    ps[i] = add_rn(zs[i], mul_rn(b, ps[i]));
  }
  __device__ void finish(const Acc3<T>&) const {
    st->rho_old = st->rho;
    st->c.iterations += 1;
    if (st->c.iterations >= st->c.max_iter) {
      st->result_norm = st->rnorm;
      finish_loop(st->c, MSG_MAX_ITER, 0);
    }
    loop_tail(st->c);
  }
};

template <typename T>
int bicg_run(sx_ctx ctx, sx_op a, const void* b, const sx_bicg_options* opt, void* x_out, sx_mem mem,
             sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m1 = opt->left_preconditioner, m2 = opt->right_preconditioner;
  SX_CHECK(check_prec(a, m1));
  SX_CHECK(check_prec(a, m2));
  sx_op at = nullptr, m1t = nullptr;
  SX_CHECK(adjoint_op(ctx, a, &at));
  (void)m1t;
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 11, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R = V(2), *RS = V(3), *Z = V(4), *ZS = V(5), *P = V(6), *PS = V(7), *Q = V(8),
    *QS = V(9), *TMP = V(10);
  if (!m1) Z = R;
  if (!m2) ZS = RS;
  BgState<T>* st = (BgState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  BgState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  SX_CHECK(launch_apply<T>(ctx, a, X, R, EpiResid<T>{B}));
  if (n > 0) SX_CUDA(cudaMemcpyAsync(RS, R, n * w, cudaMemcpyDeviceToDevice, ctx->stream));
  if (m1) SX_CHECK(launch_apply<T>(ctx, m1, R, Z, EpiPlain<T>{}));
  if (m2) SX_CHECK(launch_apply<T>(ctx, m2, RS, ZS, EpiPlain<T>{}));
  SX_CHECK(launch_vec<T>(ctx, n, BgSetup<T>{st, B, R, RS, Z, ZS, P, PS}));
  using S = BgState<T>;
  auto body = [&]() -> int {
    // q = A p (then M2), den = (p*, q)
    if (m2) {
      SX_CHECK(launch_apply<T>(ctx, a, P, TMP, EpiSkip<T, S>{st}));
      SX_CHECK(launch_apply<T>(ctx, m2, TMP, Q, EpiDots<T, S, 0>{st, PS, nullptr}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, P, Q, EpiDots<T, S, 0>{st, PS, nullptr}));
    }
    // q* = A^T p* (then M1)
    if (m1) {
      SX_CHECK(launch_apply<T>(ctx, at, PS, TMP, EpiSkip<T, S>{st}));
      SX_CHECK(launch_apply<T>(ctx, m1, TMP, QS, EpiSkip<T, S>{st}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, at, PS, QS, EpiSkip<T, S>{st}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, BgUpdate<T>{st, X, R, RS, P, Q, QS, (!m1 && !m2) ? 1 : 0}));
    if (m1 || m2) {
      SX_CHECK(apply_opt<T>(ctx, m1, R, Z, st));
      SX_CHECK(apply_opt<T>(ctx, m2, RS, ZS, st));
      SX_CHECK(launch_vec<T>(ctx, n, BgRho<T>{st, RS, Z}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, BgP<T>{st, P, PS, Z, ZS}));
    return SX_OK;
  };
  const uint64_t key[8] = {10, (uint64_t)sizeof(T), a->serial, m1 ? m1->serial : 0, m2 ? m2->serial : 0,
                           (uint64_t)n, (uint64_t)(uintptr_t)ws, at ? at->serial : 0};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m1) && op_graphable(m2), body));
  SX_CHECK(ic0_health(ctx, m1));
  SX_CHECK(ic0_health(ctx, m2));
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

// ====================================================================== CGS
template <typename T>
struct CsState {
  LoopCtl c;
  T rho, rho_new, alpha, beta, rnorm, tol, rtol, atol, result_norm;
  // sigma = (r~, v), alpha (cgs.rs:122-137)
  template <int K>
  __device__ void step(const Acc3<T>& t) {
    const T sigma = t.a;
    if (fabs(sigma) < eps10<T>()) {
      result_norm = rnorm;
      finish_loop(c, MSG_CGS_SIGMA, 0);
      return;
    }
    alpha = rho_new / sigma;
  }
  // rho_new = (r~, r) and its exit, beta (cgs.rs:85-104)
  __device__ void rho_step(T rn) {
    rho_new = rn;
    if (fabs(rn) < eps10<T>()) {
      result_norm = rnorm;
      finish_loop(c, MSG_CGS_RHO, 0);
      return;
    }
    beta = c.iterations == 0 ? T(0) : rn / rho;
  }
};

// r~ = r, u = p = q = 0, ||r||, ||b||, initial exit, first rho (cgs.rs:52-81)
template <typename T>
struct CsSetup {
  CsState<T>* st;
  const T *b, *r;
  T *rt, *u, *p, *q;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T ri = r[i];
    rt[i] = ri;
    u[i] = T(0);
    p[i] = T(0);
    q[i] = T(0);
    a.a += ri * ri;
    a.b += b[i] * b[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rnorm = sqrt(t.a);
    st->result_norm = st->rnorm;
    st->tol = fmax(st->atol, mul_rn(st->rtol, sqrt(t.b)));
    st->rho = T(1);
    if (st->rnorm <= st->tol) {
      finish_loop(st->c, MSG_CONVERGED_INITIAL, 1);
      return;
    }
    if (st->c.max_iter == 0) {
      finish_loop(st->c, MSG_MAX_ITER, 0);
      return;
    }
    st->rho_step(t.a);  // r~ == r: the products of ||r||^2
  }
};

// u = r + beta q; p = u + beta (q + beta p) (cgs.rs:106-110)
template <typename T>
struct CsUP {
  CsState<T>* st;
  const T *r, *q;
  T *u, *p;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    const T b = st->beta;
    const T ui = add_rn(r[i], mul_rn(b, q[i]));
    u[i] = ui;
    p[i] = add_rn(ui, mul_rn(b, add_rn(q[i], mul_rn(b, p[i]))));
  }
  __device__ void finish(const Acc3<T>&) const {}
};

// q = u - alpha v; u + q; with no preconditioner also x += alpha (u + q)
// (cgs.rs:140-160)
template <typename T>
struct CsQ {
  CsState<T>* st;
  const T *u, *v;
  T *q, *uq, *x;
  int fuse_x;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    const T al = st->alpha;
    const T qi = sub_rn(u[i], mul_rn(al, v[i]));
    q[i] = qi;
    const T s = add_rn(u[i], qi);
    if (fuse_x) x[i] = add_rn(x[i], mul_rn(al, s));
    else uq[i] = s;
  }
  __device__ void finish(const Acc3<T>&) const {}
};

template <typename T>
struct CsX {
  CsState<T>* st;
  T* x;
  const T* uqp;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const { x[i] = add_rn(x[i], mul_rn(st->alpha, uqp[i])); }
  __device__ void finish(const Acc3<T>&) const {}
};

// r -= alpha (v + A q^); ||r||, next rho; loop bookkeeping (cgs.rs:171-181)
template <typename T>
struct CsR {
  CsState<T>* st;
  T* r;
  const T *v, *aq, *rt;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return ended_tail(st->c); }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T ri = sub_rn(r[i], mul_rn(st->alpha, add_rn(v[i], aq[i])));
    r[i] = ri;
    a.a += ri * ri;
    a.b += rt[i] * ri;
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rho = st->rho_new;
    st->c.iterations += 1;
    st->rnorm = sqrt(t.a);
    st->result_norm = st->rnorm;
    if (st->rnorm <= st->tol) finish_loop(st->c, MSG_CONVERGED, 1);
    else if (st->c.iterations >= st->c.max_iter) finish_loop(st->c, MSG_MAX_ITER, 0);
    else st->rho_step(t.b);
    loop_tail(st->c);
  }
};

template <typename T>
int cgs_run(sx_ctx ctx, sx_op a, const void* b, const sx_bicg_options* opt, void* x_out, sx_mem mem,
            sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m = opt->right_preconditioner;
  SX_CHECK(check_prec(a, m));
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 13, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R = V(2), *RT = V(3), *U = V(4), *P = V(5), *Q = V(6), *VV = V(7), *PP = V(8),
    *UQ = V(9), *UQP = V(10), *QP = V(11), *AQ = V(12);
  if (!m) {
    PP = P;
    QP = Q;
  }
  CsState<T>* st = (CsState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  CsState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  SX_CHECK(launch_apply<T>(ctx, a, X, R, EpiResid<T>{B}));
  SX_CHECK(launch_vec<T>(ctx, n, CsSetup<T>{st, B, R, RT, U, P, Q}));
  using S = CsState<T>;
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, CsUP<T>{st, R, Q, U, P}));
    SX_CHECK(apply_opt<T>(ctx, m, P, PP, st));
    SX_CHECK(launch_apply<T>(ctx, a, PP, VV, EpiDots<T, S, 0>{st, RT, nullptr}));
    SX_CHECK(launch_vec<T>(ctx, n, CsQ<T>{st, U, VV, Q, UQ, X, m ? 0 : 1}));
    if (m) {
      SX_CHECK(apply_opt<T>(ctx, m, UQ, UQP, st));
      SX_CHECK(launch_vec<T>(ctx, n, CsX<T>{st, X, UQP}));
      SX_CHECK(apply_opt<T>(ctx, m, Q, QP, st));
    }
    SX_CHECK(launch_apply<T>(ctx, a, QP, AQ, EpiSkip<T, S>{st}));
    SX_CHECK(launch_vec<T>(ctx, n, CsR<T>{st, R, VV, AQ, RT}));
    return SX_OK;
  };
  const uint64_t key[8] = {11, (uint64_t)sizeof(T), a->serial, m ? m->serial : 0, 0, (uint64_t)n,
                           (uint64_t)(uintptr_t)ws, 0};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m), body));
  SX_CHECK(ic0_health(ctx, m));
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

// ====================================================================== QMR
template <typename T>
struct QmState {
  LoopCtl c;
  T rho, rho_old, alpha, omega, beta, rnorm, tol, rtol, atol, result_norm, nonzero;
  int first, pad;
  template <int K>
  __device__ void step(const Acc3<T>& t) {
    if constexpr (K == 0) {
      // (p~, q), alpha (qmr.rs:178-190)
      const T d = t.a;
      if (fabs(d) < eps10<T>()) {
        result_norm = rnorm;
        finish_loop(c, MSG_QMR_PQ, 0);
        return;
      }
      alpha = rho / d;
    } else {
      // omega = (t, s) / (t, t), 0 when (t, t) = 0 (qmr.rs:208-214)
      const T tt = t.b;
      omega = tt == T(0) ? T(0) : t.c / tt;
    }
  }
  // rho = (r~, r) and its exit, beta (qmr.rs:113-132)
  __device__ void rho_step(T r) {
    rho_old = rho;
    rho = r;
    if (fabs(r) < eps10<T>()) {
      result_norm = rnorm;
      finish_loop(c, MSG_QMR_RHO, 0);
      return;
    }
    beta = first ? T(0) : mul_rn(rho / rho_old, alpha / omega);
  }
};

// the initial guess is used only when some entry is non-zero (qmr.rs:65-70)
template <typename T>
struct QmNonzero {
  QmState<T>* st;
  const T* x;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += x[i] != T(0) ? T(1) : T(0); }
  __device__ void finish(const Acc3<T>& t) const { st->nonzero = t.a; }
};
template <typename T>
struct EpiQmR0 {
  const QmState<T>* st;
  const T* b;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ T out(int64_t i, T ax) const { return st->nonzero != T(0) ? sub_rn(b[i], ax) : b[i]; }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// r~ = r, p = p~ = q = q~ = 0, norms, initial exit, first rho (qmr.rs:76-132)
template <typename T>
struct QmSetup {
  QmState<T>* st;
  const T *b, *r;
  T *rt, *p, *pt, *q, *qt;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T ri = r[i];
    rt[i] = ri;
    p[i] = T(0);
    pt[i] = T(0);
    q[i] = T(0);
    qt[i] = T(0);
    a.a += ri * ri;
    a.b += b[i] * b[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->rnorm = sqrt(t.a);
    st->result_norm = st->rnorm;
    st->tol = add_rn(st->atol, mul_rn(st->rtol, sqrt(t.b)));
    st->rho = T(1);
    st->alpha = T(0);
    st->omega = T(1);
    st->first = 1;
    if (st->rnorm < st->tol) {
      finish_loop(st->c, MSG_QMR_INITIAL, 1);
      return;
    }
    if (st->c.max_iter == 0) {
      finish_loop(st->c, MSG_QMR_MAX_ITER, 0);
      return;
    }
    st->rho_step(t.a);
  }
};

// p = r + (p - q omega) beta, p~ = r~ + (p~ - q~ omega) beta; r and r~ on
// the first iteration (qmr.rs:142-162)
template <typename T>
struct QmP {
  QmState<T>* st;
  const T *r, *rt, *q, *qt;
  T *p, *pt;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const {
    if (st->first) {
      p[i] = r[i];
      pt[i] = rt[i];
      return;
    }
    const T b = st->beta, om = st->omega;
    p[i] = add_rn(r[i], mul_rn(sub_rn(p[i], mul_rn(q[i], om)), b));
    pt[i] = add_rn(rt[i], mul_rn(sub_rn(pt[i], mul_rn(qt[i], om)), b));
  }
  __device__ void finish(const Acc3<T>&) const {}
};

template <typename T>
struct QmS {
  QmState<T>* st;
  const T *r, *q;
  T* s;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const { s[i] = sub_rn(r[i], mul_rn(q[i], st->alpha)); }
  __device__ void finish(const Acc3<T>&) const {}
};

// x = (x + p^ alpha) + s^ omega; r = s - t omega; ||r|| and the exits;
// next rho (qmr.rs:217-250, 113-132)
template <typename T>
struct QmX {
  QmState<T>* st;
  T *x, *r;
  const T *pp, *sp, *s, *t, *rt;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return ended_tail(st->c); }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T al = st->alpha, om = st->omega;
    x[i] = add_rn(add_rn(x[i], mul_rn(pp[i], al)), mul_rn(sp[i], om));
    const T ri = sub_rn(s[i], mul_rn(t[i], om));
    r[i] = ri;
    a.a += ri * ri;
    a.b += rt[i] * ri;
  }
  __device__ void finish(const Acc3<T>& tot) const {
    st->rnorm = sqrt(tot.a);
    st->result_norm = st->rnorm;
    st->c.iterations += 1;
    if (st->rnorm < st->tol) finish_loop(st->c, MSG_QMR_CONVERGED, 1);
    else if (fabs(st->omega) < eps_of<T>()) finish_loop(st->c, MSG_QMR_OMEGA, 0);
    else if (st->c.iterations >= st->c.max_iter) finish_loop(st->c, MSG_QMR_MAX_ITER, 0);
    else {
      st->first = 0;
      st->rho_step(tot.b);
    }
    loop_tail(st->c);
  }
};

template <typename T>
int qmr_run(sx_ctx ctx, sx_op a, const void* b, const sx_bicg_options* opt, void* x_out, sx_mem mem,
            sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m1 = opt->left_preconditioner, m2 = opt->right_preconditioner;
  SX_CHECK(check_prec(a, m1));
  SX_CHECK(check_prec(a, m2));
  sx_op at = nullptr, m1t = nullptr, m2t = nullptr;
  SX_CHECK(adjoint_op(ctx, a, &at));
  SX_CHECK(adjoint_op(ctx, m1, &m1t));
  SX_CHECK(adjoint_op(ctx, m2, &m2t));
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 16, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R = V(2), *RT = V(3), *P = V(4), *PT = V(5), *Q = V(6), *QT = V(7), *S = V(8),
    *TT = V(9), *PP = V(10), *PTP = V(11), *SP = V(12), *TMP = V(13), *R0 = V(14), *TMP2 = V(15);
  if (!m2) {
    PP = P;
    SP = S;
  }
  if (!m1) PTP = PT;
  QmState<T>* st = (QmState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  QmState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  SX_CHECK(launch_vec<T>(ctx, n, QmNonzero<T>{st, X}));
  SX_CHECK(launch_apply<T>(ctx, a, X, m1 ? R0 : R, EpiQmR0<T>{st, B}));
  if (m1) SX_CHECK(launch_apply<T>(ctx, m1, R0, R, EpiPlain<T>{}));
  SX_CHECK(launch_vec<T>(ctx, n, QmSetup<T>{st, B, R, RT, P, PT, Q, QT}));
  using St = QmState<T>;
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, QmP<T>{st, R, RT, Q, QT, P, PT}));
    // q = M1 A M2 p, (p~, q), alpha
    SX_CHECK(apply_opt<T>(ctx, m2, P, PP, st));
    if (m1) {
      SX_CHECK(launch_apply<T>(ctx, a, PP, TMP, EpiSkip<T, St>{st}));
      SX_CHECK(launch_apply<T>(ctx, m1, TMP, Q, EpiDots<T, St, 0>{st, PT, nullptr}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, PP, Q, EpiDots<T, St, 0>{st, PT, nullptr}));
    }
    // q~ = M2^T A^T M1^T p~
    SX_CHECK(apply_opt<T>(ctx, m1t, PT, PTP, st));
    if (m2) {
      SX_CHECK(launch_apply<T>(ctx, at, PTP, TMP2, EpiSkip<T, St>{st}));
      SX_CHECK(launch_apply<T>(ctx, m2t, TMP2, QT, EpiSkip<T, St>{st}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, at, PTP, QT, EpiSkip<T, St>{st}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, QmS<T>{st, R, Q, S}));
    // t = M1 A M2 s, omega
    SX_CHECK(apply_opt<T>(ctx, m2, S, SP, st));
    if (m1) {
      SX_CHECK(launch_apply<T>(ctx, a, SP, TMP, EpiSkip<T, St>{st}));
      SX_CHECK(launch_apply<T>(ctx, m1, TMP, TT, EpiDots<T, St, 1>{st, nullptr, S}));
    } else {
      SX_CHECK(launch_apply<T>(ctx, a, SP, TT, EpiDots<T, St, 1>{st, nullptr, S}));
    }
    SX_CHECK(launch_vec<T>(ctx, n, QmX<T>{st, X, R, PP, SP, S, TT, RT}));
    return SX_OK;
  };
  const uint64_t key[8] = {12, (uint64_t)sizeof(T), a->serial, m1 ? m1->serial : 0, m2 ? m2->serial : 0,
                           (uint64_t)n, (uint64_t)(uintptr_t)ws, at ? at->serial : 0};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m1) && op_graphable(m2), body));
  SX_CHECK(ic0_health(ctx, m1));
  SX_CHECK(ic0_health(ctx, m2));
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

// =================================================================== MINRES
template <typename T>
struct MrState {
  LoopCtl c;
  T beta, oldb, dbar, epsln, phibar, cs, sn, tnorm2, qrnorm, alfa, cab, s, phi, delta, oldeps, denom, rtol,
      atol, result_norm;
  int first, error;
  // alfa = (v, y), its quotient by beta (minres.rs:171-174)
  template <int K>
  __device__ void step(const Acc3<T>& t) {
    if constexpr (K == 0) {
      alfa = t.a;
      cab = alfa / beta;
    } else {
      scalar(t.c);
    }
  }
  // beta = sqrt((r2, y)), the norm estimate and the QR rotations
  // (minres.rs:185-219)
  __device__ void scalar(T bsq) {
    oldb = beta;
    if (bsq < T(0)) {
      error = 2;
      finish_loop(c, MSG_MAX_ITER, 0);
      return;
    }
    beta = sqrt(bsq);
    tnorm2 = add_rn(add_rn(add_rn(tnorm2, mul_rn(alfa, alfa)), mul_rn(oldb, oldb)), mul_rn(beta, beta));
    oldeps = epsln;
    delta = add_rn(mul_rn(cs, dbar), mul_rn(sn, alfa));
    const T gbar = sub_rn(mul_rn(sn, dbar), mul_rn(cs, alfa));
    epsln = mul_rn(sn, beta);
    dbar = mul_rn(-cs, beta);
    const T gamma = sqrt(add_rn(mul_rn(gbar, gbar), mul_rn(beta, beta)));
    const T gc = gamma > eps_of<T>() ? gamma : eps_of<T>();
    cs = gbar / gc;
    sn = beta / gc;
    phi = mul_rn(cs, phibar);
    phibar = mul_rn(sn, phibar);
    denom = T(1) / gc;
    s = T(1) / beta;
  }
};

template <typename T>
struct MrB {
  MrState<T>* st;
  const T* b;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += b[i] * b[i]; }
  __device__ void finish(const Acc3<T>& t) const {
    // minres.rs:93-101
    if (sqrt(t.a) < st->atol) {
      st->result_norm = T(0);
      finish_loop(st->c, MSG_ZERO_RHS, 1);
    }
  }
};

// beta1^2 = (r1, M r1), r2 = r1, r1 = w = w2 = 0 (minres.rs:103-145)
template <typename T>
struct MrSetup {
  MrState<T>* st;
  T *r1, *r2, *yv, *w, *w2;
  int has_m;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T ri = r1[i];
    const T yi = has_m ? yv[i] : ri;
    if (!has_m) yv[i] = ri;
    a.a += ri * yi;
    r2[i] = ri;
    r1[i] = T(0);
    w[i] = T(0);
    w2[i] = T(0);
  }
  __device__ void finish(const Acc3<T>& t) const {
    const T b1sq = t.a;
    if (b1sq < T(0)) {
      st->error = 1;
      finish_loop(st->c, MSG_MAX_ITER, 0);
      return;
    }
    if (b1sq == T(0)) {
      st->result_norm = T(0);
      finish_loop(st->c, MSG_ZERO_RESIDUAL, 1);
      return;
    }
    const T beta1 = sqrt(b1sq);
    st->oldb = T(0);
    st->beta = beta1;
    st->dbar = T(0);
    st->epsln = T(0);
    st->phibar = beta1;
    st->cs = T(-1);
    st->sn = T(0);
    st->tnorm2 = T(0);
    st->qrnorm = beta1;
    st->s = T(1) / beta1;
    st->first = 1;
    st->result_norm = beta1;
    if (st->c.max_iter == 0) finish_loop(st->c, MSG_MAX_ITER, 0);
  }
};

template <typename T>
struct MrV {
  MrState<T>* st;
  const T* yv;
  T* v;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>&) const { v[i] = mul_rn(st->s, yv[i]); }
  __device__ void finish(const Acc3<T>&) const {}
};

// y = A v - (beta / oldb) r1 after the first step; alfa = (v, y)
// (minres.rs:164-172)
template <typename T>
struct EpiMrA {
  MrState<T>* st;
  const T *r1, *v;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ T out(int64_t i, T ax) const {
    return st->first ? ax : sub_rn(ax, mul_rn(st->beta / st->oldb, r1[i]));
  }
  __device__ void acc(int64_t i, T y, Acc3<T>& a) const { a.a += v[i] * y; }
  __device__ void finish(const Acc3<T>& t) const { st->template step<0>(t); }
};

// y -= (alfa / beta) r2; r1 = r2; r2 = y; without M also y_vec = r2 and
// (r2, y_vec) with the scalar step (minres.rs:174-189)
template <typename T>
struct MrR {
  MrState<T>* st;
  T *yn, *r1, *r2, *yv;
  int has_m;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T y = sub_rn(yn[i], mul_rn(st->cab, r2[i]));
    r1[i] = r2[i];
    r2[i] = y;
    if (!has_m) {
      yv[i] = y;
      a.c += y * y;
    }
  }
  __device__ void finish(const Acc3<T>& t) const {
    if (!has_m) st->scalar(t.c);
  }
};

// w1 = w2, w2 = w, w = (v - oldeps w1 - delta w2) denom, x += phi w, the
// convergence test on ||x|| (minres.rs:221-247)
template <typename T>
struct MrW {
  MrState<T>* st;
  const T* v;
  T *w, *w2, *x;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return ended_tail(st->c); }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T wo = w[i], w2o = w2[i];
    const T wn = mul_rn(sub_rn(sub_rn(v[i], mul_rn(st->oldeps, w2o)), mul_rn(st->delta, wo)), st->denom);
    w2[i] = wo;
    w[i] = wn;
    const T xi = add_rn(x[i], mul_rn(st->phi, wn));
    x[i] = xi;
    a.a += xi * xi;
  }
  __device__ void finish(const Acc3<T>& t) const {
    st->qrnorm = st->phibar;
    const T rnorm = st->qrnorm;
    const T anorm = sqrt(st->tnorm2);
    const T ynorm = sqrt(t.a);
    const T test1 = (ynorm == T(0) || anorm == T(0)) ? T(INFINITY) : rnorm / mul_rn(anorm, ynorm);
    st->c.iterations += 1;
    st->result_norm = rnorm;
    st->first = 0;
    if (test1 <= st->rtol || rnorm <= st->atol) finish_loop(st->c, MSG_CONVERGED, 1);
    else if (st->c.iterations >= st->c.max_iter) finish_loop(st->c, MSG_MAX_ITER, 0);
    loop_tail(st->c);
  }
};

template <typename T>
int minres_run(sx_ctx ctx, sx_op a, const void* b, const sx_minres_options* opt, void* x_out, sx_mem mem,
               sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m = opt->preconditioner;
  SX_CHECK(check_prec(a, m));
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * 9, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R1 = V(2), *R2 = V(3), *YV = V(4), *VV = V(5), *YN = V(6), *W = V(7), *W2 = V(8);
  MrState<T>* st = (MrState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  MrState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  using S = MrState<T>;
  SX_CHECK(launch_vec<T>(ctx, n, MrB<T>{st, B}));
  SX_CHECK(launch_apply<T>(ctx, a, X, R1, EpiResidSkip<T, S>{st, B}));
  if (m) SX_CHECK(launch_apply<T>(ctx, m, R1, YV, EpiSkip<T, S>{st}));
  SX_CHECK(launch_vec<T>(ctx, n, MrSetup<T>{st, R1, R2, YV, W, W2, m ? 1 : 0}));
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, MrV<T>{st, YV, VV}));
    SX_CHECK(launch_apply<T>(ctx, a, VV, YN, EpiMrA<T>{st, R1, VV}));
    SX_CHECK(launch_vec<T>(ctx, n, MrR<T>{st, YN, R1, R2, YV, m ? 1 : 0}));
    if (m) SX_CHECK(launch_apply<T>(ctx, m, R2, YV, EpiDots<T, S, 1>{st, nullptr, R2}));
    SX_CHECK(launch_vec<T>(ctx, n, MrW<T>{st, VV, W, W2, X}));
    return SX_OK;
  };
  const uint64_t key[8] = {13, (uint64_t)sizeof(T), a->serial, m ? m->serial : 0, 0, (uint64_t)n,
                           (uint64_t)(uintptr_t)ws, 0};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m), body));
  SX_CHECK(ic0_health(ctx, m));
  SX_CHECK(read_ctl(ctx, st, &h, sizeof(h)));
  if (h.error == 1) return set_error(SX_ERR_COMPUTATION, "Computation error: Indefinite preconditioner");
  if (h.error == 2) return set_error(SX_ERR_COMPUTATION, "Computation error: Non-symmetric matrix");
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

// =================================================================== LGMRES
constexpr int kLgMax = 64;  // largest inner_m

// Scalars of one outer cycle; the Hessenberg matrix, the rotations, the
// rotated right-hand side and y live in `aux` (row stride kLgMax).
template <typename T>
struct LgState {
  LoopCtl c;
  T bnorm, rn, r0n, hn, rtol, atol, result_norm;
  int active, j, k, m;
};
template <typename T>
struct LgAux {
  T h[(kLgMax + 1) * kLgMax];
  T cv[kLgMax + 1], sv[kLgMax + 1], beta[kLgMax + 2], y[kLgMax];
};

template <typename T>
struct LgB {
  LgState<T>* st;
  const T* b;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += b[i] * b[i]; }
  __device__ void finish(const Acc3<T>& t) const {
    // lgmres.rs:80-88
    st->bnorm = sqrt(t.a);
    if (st->bnorm < st->atol) {
      st->result_norm = T(0);
      finish_loop(st->c, MSG_CONVERGED, 1);
    }
  }
};

// ||r|| and the outer convergence test (lgmres.rs:108-116, :150-159); as the
// last kernel of a cycle also the cycle count and the loop condition
template <typename T>
struct LgCheck {
  LgState<T>* st;
  const T* r;
  int tail;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return tail ? ended_tail(st->c) : st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += r[i] * r[i]; }
  __device__ void finish(const Acc3<T>& t) const {
    if (tail) st->c.iterations += 1;
    st->rn = sqrt(t.a);
    st->result_norm = st->rn;
    if (st->rn < st->atol || st->rn / st->bnorm < st->rtol) finish_loop(st->c, MSG_CONVERGED, 1);
    else if (st->c.iterations >= st->c.max_iter) finish_loop(st->c, MSG_MAX_ITER, 0);
    if (tail) loop_tail(st->c);
  }
};

// inner cycle start (lgmres.rs:206-222): ||r0||, zeroed H / rotations, beta_0
template <typename T>
struct LgStart {
  LgState<T>* st;
  LgAux<T>* aux;
  const T* r;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t i, Acc3<T>& a) const { a.a += r[i] * r[i]; }
  __device__ void finish(const Acc3<T>& t) const {
    const T r0n = sqrt(t.a);
    st->r0n = r0n;
    st->j = 0;
    st->k = 0;
    const int m = st->m;
    for (int q = 0; q < (m + 1) * kLgMax; ++q) aux->h[q] = T(0);
    for (int q = 0; q <= m; ++q) aux->cv[q] = aux->sv[q] = T(0);
    for (int q = 0; q <= m + 1; ++q) aux->beta[q] = T(0);
    aux->beta[0] = r0n;
    st->active = r0n < eps_of<T>() ? 0 : 1;  // a zero correction when ||r0|| < eps
  }
};

// v_0 = r / ||r0||, or v_{j+1} = w / h_{j+1,j}
template <typename T>
struct LgScale {
  LgState<T>* st;
  const T* src;
  T* dst;
  int step;  // the step the kernel belongs to (0: v_0)
  int from_r0;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != step; }
  __device__ void elem(int64_t i, Acc3<T>&) const { dst[i] = src[i] / (from_r0 ? st->r0n : st->hn); }
  __device__ void finish(const Acc3<T>&) const {}
};

template <typename T, class S>
struct EpiLgStep {
  const S* st;
  int step;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != step; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// h_ij = (w, v_i) for i <= j, all from the unorthogonalised w (classical
// Gram-Schmidt, lgmres.rs:234-245).  Grid (gx, ceil((j+1)/8)); each block
// sums eight dots over its rows; the last block adds the partials per dot in
// block order.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_lg_dots(const LgState<T>* st, LgAux<T>* aux, int step, int64_t n,
                                                    const T* __restrict__ w, const T* __restrict__ vbase,
                                                    int64_t vstride, T* partials, unsigned int* counter) {
  if (st->c.status != ST_RUNNING || !st->active || st->j != step) return;
  const int i0 = blockIdx.y * 8;
  T acc[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) acc[t] = T(0);
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  for (int64_t r = (int64_t)blockIdx.x * kBlock + threadIdx.x; r < n; r += stride) {
    const T wr = w[r];
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (i0 + t <= step) acc[t] += wr * vbase[(int64_t)(i0 + t) * vstride + r];
  }
  __shared__ T sh[8][kWarps];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const T v = warp_sum(acc[t]);
    if (lane == 0) sh[t][wp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    T s = T(0);
    for (int q = 0; q < kWarps; ++q) s += sh[threadIdx.x][q];
    partials[(int64_t)(i0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int i = threadIdx.x; i <= step; i += kBlock) {
    T s = T(0);
    for (unsigned int bx = 0; bx < gridDim.x; ++bx) s += __ldcg(partials + (int64_t)i * gridDim.x + bx);
    aux->h[i * kLgMax + step] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// w -= sum_i h_ij v_i (per entry in i order), ||w||; then the step's scalar
// work (lgmres.rs:242-291): h_{j+1,j}, the previous rotations on column j,
// the new rotation, beta, and the inner loop's exits
template <typename T>
struct LgOrth {
  LgState<T>* st;
  LgAux<T>* aux;
  T* w;
  const T* vbase;
  int64_t vstride;
  int step;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return st->c.status != ST_RUNNING || !st->active || st->j != step; }
  __device__ void elem(int64_t r, Acc3<T>& a) const {
    T x = w[r];
    for (int i = 0; i <= step; ++i) x = sub_rn(x, mul_rn(aux->h[i * kLgMax + step], vbase[(int64_t)i * vstride + r]));
    w[r] = x;
    a.a += x * x;
  }
  __device__ void finish(const Acc3<T>& t) const {
    const int j = step;
    const T eps = eps_of<T>();
    T* H = aux->h;
    auto h = [&](int i, int c) -> T& { return H[i * kLgMax + c]; };
    const T hn = sqrt(t.a);
    if (!(hn > eps)) {
      st->k = j + 1;
      st->active = 0;
      return;
    }
    h(j + 1, j) = hn;
    st->hn = hn;
    for (int i = 0; i < j; ++i) {
      const T temp = add_rn(mul_rn(aux->cv[i], h(i, j)), mul_rn(aux->sv[i], h(i + 1, j)));
      h(i + 1, j) = add_rn(mul_rn(-aux->sv[i], h(i, j)), mul_rn(aux->cv[i], h(i + 1, j)));
      h(i, j) = temp;
    }
    const T hjj = h(j, j), hj1 = h(j + 1, j);
    const T rho = sqrt(add_rn(mul_rn(hjj, hjj), mul_rn(hj1, hj1)));
    if (rho > eps) {
      aux->cv[j] = hjj / rho;
      aux->sv[j] = hj1 / rho;
      h(j, j) = add_rn(mul_rn(aux->cv[j], hjj), mul_rn(aux->sv[j], hj1));
      h(j + 1, j) = T(0);
      aux->beta[j + 1] = mul_rn(-aux->sv[j], aux->beta[j]);
      aux->beta[j] = mul_rn(aux->cv[j], aux->beta[j]);
      st->k = j + 1;
      if (fabs(aux->beta[j + 1]) < T(1e-10) || j + 1 >= st->m) st->active = 0;
      else st->j = j + 1;
    } else {
      st->k = j;
      st->active = 0;
    }
  }
};

// y from the triangular system (lgmres.rs:300-312), one thread
template <typename T>
__global__ void k_lg_back(LgState<T>* st, LgAux<T>* aux) {
  if (st->c.status != ST_RUNNING || threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = st->k;
  const T eps = eps_of<T>();
  for (int i = k - 1; i >= 0; --i) {
    T yi = aux->beta[i];
    for (int q = i + 1; q < k; ++q) yi = sub_rn(yi, mul_rn(aux->h[i * kLgMax + q], aux->y[q]));
    const T hii = aux->h[i * kLgMax + i];
    aux->y[i] = fabs(hii) > eps ? yi / hii : T(0);
  }
}

// x += sum_i y_i v_i, the inner sum in i order from zero (lgmres.rs:315-320,
// :131-134)
template <typename T>
struct LgX {
  LgState<T>* st;
  const LgAux<T>* aux;
  T* x;
  const T* vbase;
  int64_t vstride;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return st->c.status != ST_RUNNING; }
  __device__ void elem(int64_t r, Acc3<T>&) const {
    const int k = st->k;
    T s = T(0);
    for (int i = 0; i < k; ++i) s = add_rn(s, mul_rn(aux->y[i], vbase[(int64_t)i * vstride + r]));
    x[r] = add_rn(x[r], s);
  }
  __device__ void finish(const Acc3<T>&) const {}
};

template <typename T>
int lgmres_run(sx_ctx ctx, sx_op a, const void* b, const sx_lgmres_options* opt, void* x_out, sx_mem mem,
               sx_iter_result* res) {
  const int64_t n = a->nrows;
  sx_op m = opt->preconditioner;
  SX_CHECK(check_prec(a, m));
  const int mm = (int)opt->inner_m;
  const size_t w = sizeof(T);
  const size_t vb = align_up((size_t)std::max<int64_t>(n, 1) * w, 256);
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(vec_grid(ctx, n), (int64_t)ctx->num_sms * 4));
  const size_t aux_b = align_up(sizeof(LgAux<T>), 256);
  const size_t part_b = align_up((size_t)gx * (kLgMax + 8) * w, 256);
  void *ws = nullptr, *dstate = nullptr;
  SX_CHECK(ws_get(ctx, vb * (size_t)(6 + mm + 1) + aux_b + part_b, &ws, &dstate));
  auto V = [&](int i) { return (T*)((char*)ws + (size_t)i * vb); };
  T *B = V(0), *X = V(1), *R = V(2), *R0 = V(3), *W = V(4), *TMP = V(5), *VB = V(6);
  LgAux<T>* aux = (LgAux<T>*)((char*)ws + vb * (size_t)(6 + mm + 1));
  T* part = (T*)((char*)aux + aux_b);
  const int64_t vstride = (int64_t)(vb / w);
  if (!m) R = R0;
  LgState<T>* st = (LgState<T>*)dstate;
  SX_CHECK(vec_in(ctx, B, b, n * w, mem));
  if (opt->x0) SX_CHECK(vec_in(ctx, X, opt->x0, n * w, mem));
  else if (n > 0) SX_CUDA(cudaMemsetAsync(X, 0, n * w, ctx->stream));
  LgState<T> h;
  std::memset(&h, 0, sizeof(h));
  h.c.max_iter = opt->max_iter;
  h.rtol = (T)opt->rtol;
  h.atol = (T)opt->atol;
  h.m = mm;
  SX_CHECK(write_bytes(ctx, st, &h, sizeof(h)));
  ReduceArea ra;
  SX_CHECK(ctx_reduce_area(ctx, std::max<int64_t>((n + kBlock - 1) / kBlock, vec_grid(ctx, n)) + 8, &ra));
  using S = LgState<T>;
  SX_CHECK(launch_vec<T>(ctx, n, LgB<T>{st, B}));
  auto residual = [&]() -> int {
    SX_CHECK(launch_apply<T>(ctx, a, X, R0, EpiResidSkip<T, S>{st, B}));
    if (m) SX_CHECK(launch_apply<T>(ctx, m, R0, R, EpiSkip<T, S>{st}));
    return SX_OK;
  };
  SX_CHECK(residual());
  SX_CHECK(launch_vec<T>(ctx, n, LgCheck<T>{st, R, 0}));
  auto body = [&]() -> int {
    SX_CHECK(launch_vec<T>(ctx, n, LgStart<T>{st, aux, R}));
    SX_CHECK(launch_vec<T>(ctx, n, LgScale<T>{st, R, VB, 0, 1}));
    for (int j = 0; j < mm; ++j) {
      T* vj = VB + (int64_t)j * vstride;
      if (m) {
        SX_CHECK(launch_apply<T>(ctx, a, vj, TMP, EpiLgStep<T, S>{st, j}));
        SX_CHECK(launch_apply<T>(ctx, m, TMP, W, EpiLgStep<T, S>{st, j}));
      } else {
        SX_CHECK(launch_apply<T>(ctx, a, vj, W, EpiLgStep<T, S>{st, j}));
      }
      dim3 grid((unsigned)gx, (unsigned)((j + 1 + 7) / 8));
      if (n > 0) {
        k_lg_dots<T><<<grid, kBlock, 0, ctx->stream>>>(st, aux, j, n, W, VB, vstride, part, ra.counter);
        ctx->launches++;
        SX_CUDA(cudaGetLastError());
      }
      SX_CHECK(launch_vec<T>(ctx, n, LgOrth<T>{st, aux, W, VB, vstride, j}));
      if (j + 1 < mm) SX_CHECK(launch_vec<T>(ctx, n, LgScale<T>{st, W, VB + (int64_t)(j + 1) * vstride, j + 1, 0}));
    }
    k_lg_back<T><<<1, 32, 0, ctx->stream>>>(st, aux);
    ctx->launches++;
    SX_CUDA(cudaGetLastError());
    SX_CHECK(launch_vec<T>(ctx, n, LgX<T>{st, aux, X, VB, vstride}));
    SX_CHECK(residual());
    SX_CHECK(launch_vec<T>(ctx, n, LgCheck<T>{st, R, 1}));
    return SX_OK;
  };
  const uint64_t key[8] = {14, (uint64_t)sizeof(T), a->serial, m ? m->serial : 0, (uint64_t)mm, (uint64_t)n,
                           (uint64_t)(uintptr_t)ws, (uint64_t)gx};
  SX_CHECK(run_loop(ctx, st, key, op_graphable(a) && op_graphable(m), body));
  SX_CHECK(ic0_health(ctx, m));
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

// Rust's `{}` formatting of a float: the shortest decimal that reads back to
// the same value, never in exponent form ("0.0001", "1e21" as
// "1000000000000000000000"), "NaN", "inf", "-inf".
template <typename F>
std::string rust_display(F v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v < 0 ? "-inf" : "inf";
  char buf[512];
  auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::fixed);
  return std::string(buf, r.ptr);
}

}  // namespace
}  // namespace sx

using namespace sx;

extern "C" {

void sx_bicg_options_default(sx_bicg_options* o) {
  o->max_iter = 1000;
  o->rtol = 1e-8;
  o->atol = 1e-12;
  o->x0 = nullptr;
  o->left_preconditioner = nullptr;
  o->right_preconditioner = nullptr;
}
void sx_minres_options_default(sx_minres_options* o) {
  o->max_iter = 1000;
  o->rtol = 1e-8;
  o->atol = 1e-12;
  o->x0 = nullptr;
  o->preconditioner = nullptr;
}
void sx_lgmres_options_default(sx_lgmres_options* o) {
  o->max_iter = 500;
  o->rtol = 1e-8;
  o->atol = 1e-8;
  o->inner_m = 30;
  o->outer_k = 3;
  o->x0 = nullptr;
  o->preconditioner = nullptr;
}

int sx_bicg(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt, void* x_out,
            sx_mem mem, sx_iter_result* res) {
  SX_CHECK(solver_checks(ctx, a, b, b_len, x_out, "BiCG"));
  sx_bicg_options d;
  if (!opt) {
    sx_bicg_options_default(&d);
    opt = &d;
  }
  int rc = a->dtype == SX_F64 ? bicg_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : bicg_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_cgs(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt, void* x_out,
           sx_mem mem, sx_iter_result* res) {
  SX_CHECK(solver_checks(ctx, a, b, b_len, x_out, "CGS"));
  sx_bicg_options d;
  if (!opt) {
    sx_bicg_options_default(&d);
    opt = &d;
  }
  int rc = a->dtype == SX_F64 ? cgs_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : cgs_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_qmr(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_bicg_options* opt, void* x_out,
           sx_mem mem, sx_iter_result* res) {
  if (!ctx || !a) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx/operator");
  // qmr.rs:53-59: DimensionMismatch{expected: b.len(), found: rows}
  if ((uint64_t)a->nrows != b_len || (uint64_t)a->ncols != b_len)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(b_len) + ", found " +
                         std::to_string(a->nrows),
                     b_len, (uint64_t)a->nrows);
  if (b_len > 0 && (!b || !x_out)) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null b/x");
  SX_CUDA(cudaSetDevice(ctx->device));
  sx_bicg_options d;
  if (!opt) {
    sx_bicg_options_default(&d);
    opt = &d;
  }
  int rc = a->dtype == SX_F64 ? qmr_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : qmr_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

static int square_then_len(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, void* x_out) {
  if (!ctx || !a) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null ctx/operator");
  // minres.rs:75-87, lgmres.rs:66-78
  if (a->nrows != a->ncols)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a->nrows) + ", found " +
                         std::to_string(a->ncols),
                     (uint64_t)a->nrows, (uint64_t)a->ncols);
  if (b_len != (uint64_t)a->ncols)
    return set_error(SX_ERR_DIMENSION_MISMATCH,
                     "Dimension mismatch: expected " + std::to_string(a->ncols) + ", found " +
                         std::to_string(b_len),
                     (uint64_t)a->ncols, b_len);
  if (b_len > 0 && (!b || !x_out)) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null b/x");
  SX_CUDA(cudaSetDevice(ctx->device));
  return SX_OK;
}

int sx_minres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_minres_options* opt, void* x_out,
              sx_mem mem, sx_iter_result* res) {
  SX_CHECK(square_then_len(ctx, a, b, b_len, x_out));
  sx_minres_options d;
  if (!opt) {
    sx_minres_options_default(&d);
    opt = &d;
  }
  int rc = a->dtype == SX_F64 ? minres_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : minres_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_lgmres(sx_ctx ctx, sx_op a, const void* b, uint64_t b_len, const sx_lgmres_options* opt, void* x_out,
              sx_mem mem, sx_iter_result* res) {
  SX_CHECK(square_then_len(ctx, a, b, b_len, x_out));
  sx_lgmres_options d;
  if (!opt) {
    sx_lgmres_options_default(&d);
    opt = &d;
  }
  if (opt->inner_m < 1 || opt->inner_m > (uint64_t)kLgMax)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: inner_m must be in 1..=64");
  int rc = a->dtype == SX_F64 ? lgmres_run<double>(ctx, a, b, opt, x_out, mem, res)
                              : lgmres_run<float>(ctx, a, b, opt, x_out, mem, res);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_iter_message(const sx_iter_result* res, int dtype, char* buf, uint64_t len) {
  if (!res || !buf || len == 0) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  std::string s;
  const std::string r = dtype == SX_F32 ? rust_display<float>((float)res->residual_norm)
                                        : rust_display<double>(res->residual_norm);
  if (res->message == MSG_QMR_CONVERGED)
    s = "Converged in " + std::to_string(res->iterations) + " iterations";
  else if (res->message == MSG_QMR_MAX_ITER)
    s = "Did not converge in " + std::to_string(res->iterations) + " iterations. Residual: " + r;
  else
    s = sx_message_string(res->message);
  std::snprintf(buf, (size_t)len, "%s", s.c_str());
  return SX_OK;
}

}  // extern "C"
