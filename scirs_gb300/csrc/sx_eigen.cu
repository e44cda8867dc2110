// Eigenpairs of symmetric CSR operators: power_iteration and lanczos of
// scirs2-sparse (src/linalg/eigen.rs:124-494).
//
// The vector work runs on the device: the symmetric SpMV (the merged-row
// form that reproduces sym_csr_matvec), and one fused kernel per
// Gram-Schmidt step that subtracts the previous projection and forms the
// next dot product, with the projections kept in device memory so the
// reorthogonalisation of a step needs no host round trip.  The host reads
// two scalars per step and runs the reference's scalar logic: the loop
// tests, the tridiagonal eigensolver (QL for more than three rows, closed
// forms below), Ritz coefficients and residuals.  Sums on the device are
// tree reductions, so results agree with the reference's sequential folds
// to rounding, not bit for bit.
//
// The reference's behaviour is kept as it is, including:
//   - lanczos keeps the first beta for every step (eigen.rs:441-443 binds a
//     new variable), so each Lanczos vector is w / beta_1 and every
//     off-diagonal entry of the tridiagonal matrix is beta_1;
//   - its QL sweep leaves the loop after one sweep for l >= 1
//     (eigen.rs:617-620);
//   - Ritz vectors and the Kaniel-Paige bound read the eigenvector list as
//     eigvecs[j][k] (eigen.rs:459, :485);
//   - solve_cubic's trigonometric branch (eigen.rs:930-940) takes
//     acos(+b / ...).
// Where the reference panics (an index past the end of those lists, or a
// subspace of size 0) these functions return a ComputationError naming it.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "sx_internal.h"
#include "sx_kernels.cuh"
#include "sx_launch.cuh"

namespace sx {
namespace {

// ------------------------------------------------------------ device bodies
// out[0] = x.y, out[1] = y.y
template <typename T>
struct EgDot2 {
  const T *x, *y;
  T* out;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    a.a += x[i] * y[i];
    a.b += y[i] * y[i];
  }
  __device__ void finish(const Acc3<T>& t) const {
    out[0] = t.a;
    out[1] = t.b;
  }
};

// One Gram-Schmidt step: w -= s_prev v_prev (when v_prev is set), then
// out = v . w with the updated w
template <typename T>
struct EgMgs {
  T* w;
  const T* vprev;
  const T* sprev;  // device scalar
  const T* v;
  T* out;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    T wi = w[i];
    if (vprev) {
      wi = sub_rn(wi, mul_rn(*sprev, vprev[i]));
      w[i] = wi;
    }
    a.a += v[i] * wi;
  }
  __device__ void finish(const Acc3<T>& t) const { *out = t.a; }
};

// w -= s v (s on the device), out = w . w
template <typename T>
struct EgAxpyNorm {
  T* w;
  const T* v;
  const T* s;
  T* out;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T wi = sub_rn(w[i], mul_rn(*s, v[i]));
    w[i] = wi;
    a.a += wi * wi;
  }
  __device__ void finish(const Acc3<T>& t) const { *out = t.a; }
};

// dst = src / s (host scalar)
template <typename T>
struct EgScale {
  const T* src;
  T* dst;
  T s;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>&) const { dst[i] = src[i] / s; }
  __device__ void finish(const Acc3<T>&) const {}
};
template <typename T>
struct EgCopy {
  const T* src;
  T* dst;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>&) const { dst[i] = src[i]; }
  __device__ void finish(const Acc3<T>&) const {}
};
// out = sum (ax - lambda x)^2
template <typename T>
struct EgResid {
  const T *ax, *x;
  T lambda;
  T* out;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>& a) const {
    const T r = sub_rn(ax[i], mul_rn(lambda, x[i]));
    a.a += r * r;
  }
  __device__ void finish(const Acc3<T>& t) const { *out = t.a; }
};
// column k of the row-major n x cols matrix
template <typename T>
struct EgColumn {
  const T* m;
  int64_t cols, k;
  T* dst;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ void elem(int64_t i, Acc3<T>&) const { dst[i] = m[i * cols + k]; }
  __device__ void finish(const Acc3<T>&) const {}
};

// Ritz vectors: out[i * cols + k] = sum_j coef[j * cols + k] V[j][i] for
// j < nj, summed in j order from zero (eigen.rs:453-465)
template <typename T>
__global__ void k_ritz(const T* __restrict__ V, int64_t n, int64_t ldv, int nj, const T* __restrict__ coef,
                       int cols, T* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    for (int k = 0; k < cols; ++k) {
      T s = T(0);
      for (int j = 0; j < nj; ++j) s = add_rn(s, mul_rn(coef[j * cols + k], V[(int64_t)j * ldv + i]));
      out[i * cols + k] = s;
    }
}

// ------------------------------------------------------ host scalar logic
int err_arg(const char* s) { return set_error(SX_ERR_INVALID_ARGUMENT, std::string("Invalid argument: ") + s); }
int err_dim(uint64_t expected, uint64_t found) {
  return set_error(SX_ERR_DIMENSION_MISMATCH,
                   "Dimension mismatch: expected " + std::to_string(expected) + ", found " + std::to_string(found),
                   expected, found);
}
int err_panic(const std::string& what) { return set_error(SX_ERR_COMPUTATION, "Computation error: panic: " + what); }

// solve_cubic, eigen.rs:890-952 (x^3 + p x^2 + q x + r)
template <typename T>
std::vector<T> cubic_roots(T p, T q, T r) {
  const T p3 = p / T(3.0);
  const T a = q - p * p3;
  const T b = r + p3 * (T(2.0) * (p3 * p3) - q);
  const T disc = T(4.0) * a * a * a + T(27.0) * b * b;
  if (disc == T(0)) {
    if (a == T(0)) return {-p3, -p3, -p3};
    const T x1 = T(3.0) * b / a, x2 = -x1 / T(2.0);
    return {x1 - p3, x2 - p3, x2 - p3};
  }
  if (disc > T(0)) {
    const T h = std::sqrt(disc) * T(0.5);
    const T c1 = (-b + h) / T(2.0), c2 = (-b - h) / T(2.0);
    const T third = (T)(1.0 / 3.0);
    auto cbrt_signed = [&](T c) { return std::pow(std::fabs(c), third) * (c >= T(0) ? T(1) : T(-1)); };
    return {cbrt_signed(c1) + cbrt_signed(c2) - p3};
  }
  const T ps = std::sqrt(-a / T(3.0));
  const T theta = std::acos(b / (T(2.0) * ps * ps * ps));
  std::vector<T> out;
  for (int k = 0; k < 3; ++k)
    out.push_back(T(2.0) * ps * std::cos((T)(3.141592653589793 * (2.0 * k) / 3.0) - theta / T(3.0)) - p3);
  return out;
}

// eigenvalues (descending) and the eigenvector list of the tridiagonal
// matrix (alpha, beta), first num of them
template <typename T>
struct TriEig {
  std::vector<T> vals;
  std::vector<std::vector<T>> vecs;  // vecs[k]: eigenvector k
};

// (A - lambda I) v = 0 for the 3 x 3 tridiagonal matrix by elimination on
// the row of largest norm (eigen.rs:767-860)
template <typename T>
std::vector<T> null_vector3(T a, T b, T c, T d, T e, T lambda, size_t num) {
  T m[3][3] = {{a - lambda, d, T(0)}, {d, b - lambda, e}, {T(0), e, c - lambda}};
  T rn[3];
  for (int r = 0; r < 3; ++r) rn[r] = std::sqrt(m[r][0] * m[r][0] + m[r][1] * m[r][1] + m[r][2] * m[r][2]);
  std::vector<T> v(3, T(0));
  if (rn[0] >= rn[1] && rn[0] >= rn[2] && rn[0] != T(0)) {
    const T s = T(1) / rn[0];
    for (int q = 0; q < 3; ++q) m[0][q] = m[0][q] * s;
    T f = m[1][0] / m[0][0];
    m[1][1] = m[1][1] - f * m[0][1];
    m[1][2] = m[1][2] - f * m[0][2];
    f = m[2][0] / m[0][0];
    m[2][1] = m[2][1] - f * m[0][1];
    m[2][2] = m[2][2] - f * m[0][2];
    v[2] = T(1);
    v[1] = -m[1][2] * v[2] / m[1][1];
    v[0] = -(m[0][1] * v[1] + m[0][2] * v[2]) / m[0][0];
  } else if (rn[1] >= rn[0] && rn[1] >= rn[2] && rn[1] != T(0)) {
    const T s = T(1) / rn[1];
    for (int q = 0; q < 3; ++q) m[1][q] = m[1][q] * s;
    T f = m[0][1] / m[1][1];
    m[0][0] = m[0][0] - f * m[1][0];
    m[0][2] = m[0][2] - f * m[1][2];
    f = m[2][1] / m[1][1];
    m[2][0] = m[2][0] - f * m[1][0];
    m[2][2] = m[2][2] - f * m[1][2];
    v[2] = T(1);
    v[0] = -m[0][2] * v[2] / m[0][0];
    v[1] = -(m[1][0] * v[0] + m[1][2] * v[2]) / m[1][1];
  } else if (rn[2] != T(0)) {
    const T s = T(1) / rn[2];
    for (int q = 0; q < 3; ++q) m[2][q] = m[2][q] * s;
    T f = m[0][2] / m[2][2];
    m[0][0] = m[0][0] - f * m[2][0];
    m[0][1] = m[0][1] - f * m[2][1];
    f = m[1][2] / m[2][2];
    m[1][0] = m[1][0] - f * m[2][0];
    m[1][1] = m[1][1] - f * m[2][1];
    v[0] = T(1);
    v[1] = -m[1][0] * v[0] / m[1][1];
    v[2] = -(m[2][0] * v[0] + m[2][1] * v[1]) / m[2][2];
  } else {
    v[num >= 1 ? 0 : 2] = T(1);  // the reference's chain reaches only these two
  }
  const T nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (nv != T(0))
    for (auto& t : v) t = t / nv;
  return v;
}

// solve_small_tridiagonal, eigen.rs:650-886
template <typename T>
int tri_small(const std::vector<T>& al, const std::vector<T>& be, size_t num, TriEig<T>& out) {
  out.vals.clear();
  out.vecs.clear();
  const size_t n = al.size();
  if (n == 1) {
    out.vals = {al[0]};
    out.vecs = {{T(1)}};
    return SX_OK;
  }
  if (n == 2) {
    const T a = al[0], b = al[1], c = be[0];
    const T tr = a + b, det = a * b - c * c;
    const T disc = std::sqrt(tr * tr - T(4.0) * det);
    T l1 = (tr + disc) * T(0.5), l2 = (tr - disc) * T(0.5);
    if (!(l1 >= l2)) std::swap(l1, l2);
    std::vector<T> v1, v2;
    if (c != T(0)) {
      v1 = {c, l1 - a};
      v2 = {c, l2 - a};
      for (auto* v : {&v1, &v2}) {
        const T nv = std::sqrt((*v)[0] * (*v)[0] + (*v)[1] * (*v)[1]);
        if (nv != T(0)) { (*v)[0] = (*v)[0] / nv; (*v)[1] = (*v)[1] / nv; }
      }
    } else if (a >= b) {
      v1 = {T(1), T(0)};
      v2 = {T(0), T(1)};
    } else {
      v1 = {T(0), T(1)};
      v2 = {T(1), T(0)};
    }
    out.vals = {l1, l2};
    out.vecs = {v1, v2};
    out.vals.resize(std::min<size_t>(2, num));
    out.vecs.resize(std::min<size_t>(2, num));
    return SX_OK;
  }
  const T a = al[0], b = al[1], c = al[2], d = be[0], e = be[1];
  const T p = -(a + b + c);
  const T q = a * b + a * c + b * c - d * d - e * e;
  const T r = -(a * b * c - a * e * e - c * d * d);
  std::vector<T> roots = cubic_roots<T>(p, q, r);
  std::stable_sort(roots.begin(), roots.end(), [](T x, T y) { return x > y; });
  const size_t take = std::min<size_t>(num, 3);
  if (take > roots.size()) return err_panic("slice index out of range for the cubic's roots");
  for (size_t t = 0; t < take; ++t) out.vecs.push_back(null_vector3<T>(a, b, c, d, e, roots[t], num));
  roots.resize(std::min(roots.size(), num));
  out.vals = roots;
  return SX_OK;
}

// solve_tridiagonal_eigenproblem, eigen.rs:512-646
template <typename T>
int tri_eig(const std::vector<T>& al, const std::vector<T>& be, size_t num, TriEig<T>& out) {
  const size_t n = al.size();
  if (n == 0) return set_error(SX_ERR_VALUE, "Value error: Empty tridiagonal matrix");
  if (be.size() != n - 1) return err_dim(n - 1, be.size());
  if (n <= 3) return tri_small<T>(al, be, num, out);
  std::vector<T> d = al, e = be;
  e.push_back(T(0));
  std::vector<T> z(n * n, T(0));  // z[row * n + col]
  for (size_t i = 0; i < n; ++i) z[i * n + i] = T(1);
  const T small = (T)1e-12;
  for (size_t l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      size_t m = l;
      while (m < n - 1 && !(std::fabs(e[m]) <= small * (std::fabs(d[m]) + std::fabs(d[m + 1])))) ++m;
      if (m == l) break;
      if (iter >= 30)
        return set_error(SX_ERR_ITERATIVE_SOLVER_FAILURE, "Iterative solver failure: QL algorithm did not converge");
      T g = (d[l + 1] - d[l]) * T(0.5) / e[l];
      const T r = std::sqrt(g * g + T(1));
      g = d[m] - d[l] + e[l] / (g + (g >= T(0) ? r : -r));
      T s = T(1), c = T(1), p = T(0);
      size_t i = m - 1;
      while (i >= l && i < n) {
        const T f = s * e[i], b = c * e[i];
        const T rr = std::sqrt(f * f + g * g);
        e[i + 1] = rr;
        if (rr == T(0)) {
          d[i + 1] = d[i + 1] - p;
          e[m] = T(0);
          break;
        }
        s = f / rr;
        c = g / rr;
        p = s * (d[i] - d[i + 1]) + c * b;
        d[i + 1] = d[i + 1] + p;
        g = c * s - b;
        for (size_t k = 0; k < n; ++k) {
          const T t = z[k * n + i + 1];
          z[k * n + i + 1] = s * z[k * n + i] + c * t;
          z[k * n + i] = c * z[k * n + i] - s * t;
        }
        if (i == 0) break;
        --i;
      }
      if ((int32_t)i < (int32_t)l || i >= n) break;  // one sweep for l >= 1
      // (the reference's r == 0 branch cannot run: r >= 1)
    }
  }
  std::vector<size_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return d[x] > d[y]; });
  out.vals.clear();
  out.vecs.clear();
  for (size_t k = 0; k < std::min(num, n); ++k) {
    out.vals.push_back(d[idx[k]]);
    std::vector<T> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = z[i * n + idx[k]];
    out.vecs.push_back(v);
  }
  return SX_OK;
}

// ------------------------------------------------------------- workspaces
template <typename T>
struct EgWork {
  sx_ctx ctx;
  T* sc = nullptr;  // device scalars
  std::vector<void*> bufs;
  ~EgWork() {
    if (ctx) cudaStreamSynchronize(ctx->stream);
    for (void* p : bufs) dev_free(p);
    dev_free(sc);
  }
  int alloc(T** p, int64_t count) {
    void* q = nullptr;
    SX_CHECK(dev_alloc(&q, (size_t)std::max<int64_t>(count, 1) * sizeof(T)));
    bufs.push_back(q);
    *p = (T*)q;
    return SX_OK;
  }
  // host copies of device scalars [0, count)
  int read(T* host, int count) {
    SX_CUDA(cudaMemcpyAsync(host, sc, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "eigen scalars", __FILE__, __LINE__);
    return SX_OK;
  }
};

template <typename T>
int apply(sx_ctx ctx, sx_op a, const T* x, T* y) {
  return launch_apply<T, EpiPlain<T>, true>(ctx, a, x, y, EpiPlain<T>{});
}

template <typename T>
int upload_start(sx_ctx ctx, const void* x0, int64_t n, sx_mem mem, T* dst) {
  if (x0) {
    if (n > 0)
      SX_CUDA(cudaMemcpyAsync(dst, x0, n * sizeof(T),
                              mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  } else {
    SX_CUDA(cudaMemsetAsync(dst, 0, std::max<int64_t>(n, 1) * sizeof(T), ctx->stream));
    const T one = T(1);
    if (n > 0) SX_CUDA(cudaMemcpyAsync(dst, &one, sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    SX_CUDA(cudaStreamSynchronize(ctx->stream));  // `one` lives on this frame
  }
  return SX_OK;
}

template <typename T>
int download(sx_ctx ctx, const T* src, int64_t count, sx_mem mem, void* dst) {
  if (count > 0)
    SX_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T),
                            mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
  return SX_OK;
}

// power_iteration, eigen.rs:124-293
template <typename T>
int power_impl(sx_ctx ctx, sx_op a, const sx_power_options& o, const void* x0, sx_mem mem, T* lambda_out,
               void* vec_out, T* resid_out, sx_eigen_result* res) {
  const int64_t n = a->nrows;
  EgWork<T> W{ctx};
  T *x = nullptr, *y = nullptr;
  SX_CHECK(dev_alloc((void**)&W.sc, 16 * sizeof(T)));
  SX_CHECK(W.alloc(&x, n));
  SX_CHECK(W.alloc(&y, n));
  SX_CHECK(upload_start<T>(ctx, x0, n, mem, x));
  T h[2];
  if (o.normalize) {
    SX_CHECK(launch_vec<T>(ctx, n, EgDot2<T>{x, x, W.sc}));
    SX_CHECK(W.read(h, 2));
    const T nrm = std::sqrt(h[1]);
    if (nrm != T(0)) SX_CHECK(launch_vec<T>(ctx, n, EgScale<T>{x, x, nrm}));
  }
  const T tol = (T)o.tol;
  T lambda = T(0), prev = T(0);
  bool conv = false;
  uint64_t it = 0;
  while (it < o.max_iter) {
    SX_CHECK(apply<T>(ctx, a, x, y));
    SX_CHECK(launch_vec<T>(ctx, n, EgDot2<T>{x, y, W.sc}));  // x.y, y.y
    SX_CHECK(W.read(h, 2));
    if (o.normalize) {
      lambda = h[0];
      if (std::fabs(lambda - prev) < tol) { conv = true; break; }
      const T nrm = std::sqrt(h[1]);
      if (nrm != T(0)) SX_CHECK(launch_vec<T>(ctx, n, EgScale<T>{y, x, nrm}));
    } else {
      SX_CHECK(launch_vec<T>(ctx, n, EgCopy<T>{y, x}));
      const T nx = std::sqrt(h[1]);  // ||x|| of the new x = y
      if (nx != T(0)) lambda = h[0] / (nx * nx);
      if (std::fabs(lambda - prev) < tol) { conv = true; break; }
    }
    prev = lambda;
    ++it;
  }
  SX_CHECK(apply<T>(ctx, a, x, y));
  SX_CHECK(launch_vec<T>(ctx, n, EgResid<T>{y, x, lambda, W.sc}));
  SX_CHECK(W.read(h, 1));
  *lambda_out = lambda;
  *resid_out = std::sqrt(h[0]);
  if (vec_out) SX_CHECK(download<T>(ctx, x, n, mem, vec_out));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  res->iterations = it;
  res->converged = conv ? 1 : 0;
  res->num_eigenvalues = 1;
  res->num_columns = 1;
  return SX_OK;
}

// lanczos, eigen.rs:295-494
template <typename T>
int lanczos_impl(sx_ctx ctx, sx_op a, const sx_lanczos_options& o, const void* v0, sx_mem mem, T* vals_out,
                 void* vecs_out, T* resid_out, sx_eigen_result* res) {
  const int64_t n = a->nrows;
  const uint64_t sub = std::min<uint64_t>(o.max_subspace_size, (uint64_t)n);
  const uint64_t num = std::min<uint64_t>(o.num_eigenvalues, sub);
  if (sub == 0) return err_panic("capacity overflow (subspace size 0)");
  if (sub > 4096) return err_arg("max_subspace_size above 4096");
  EgWork<T> W{ctx};
  T *V = nullptr, *w = nullptr;
  SX_CHECK(dev_alloc((void**)&W.sc, (sub + 8) * sizeof(T)));
  // basis vectors one padded stride apart (a multiple of 32 elements), so
  // that every vector starts 256-byte aligned like the other work vectors
  const int64_t ldv = (n + 31) / 32 * 32;
  SX_CHECK(W.alloc(&V, (int64_t)sub * ldv));
  SX_CHECK(W.alloc(&w, n));
  SX_CHECK(upload_start<T>(ctx, v0, n, mem, V));
  T h[2];
  // v = v / ||v||
  SX_CHECK(launch_vec<T>(ctx, n, EgDot2<T>{V, V, W.sc}));
  SX_CHECK(W.read(h, 2));
  const T nrm = std::sqrt(h[1]);
  if (nrm != T(0)) SX_CHECK(launch_vec<T>(ctx, n, EgScale<T>{V, V, nrm}));
  std::vector<T> alpha, beta;
  // w = A v, alpha_0 = v.w, w -= alpha_0 v, beta_1 = ||w||
  SX_CHECK(apply<T>(ctx, a, V, w));
  SX_CHECK(launch_vec<T>(ctx, n, EgDot2<T>{V, w, W.sc}));
  SX_CHECK(W.read(h, 1));
  alpha.push_back(h[0]);
  SX_CHECK(launch_vec<T>(ctx, n, EgAxpyNorm<T>{w, V, W.sc, W.sc + 1}));
  SX_CHECK(W.read(h, 2));
  const T beta1 = std::sqrt(h[1]);  // kept for every step, as the reference does
  uint64_t it = 1, nv = 1;
  bool conv = false;
  TriEig<T> te;
  const T tol = (T)o.tol;
  while (it < o.max_iter && alpha.size() < sub) {
    if (beta1 == T(0)) break;
    beta.push_back(beta1);
    T* vn = V + (int64_t)nv * ldv;
    SX_CHECK(launch_vec<T>(ctx, n, EgScale<T>{w, vn, beta1}));
    ++nv;
    SX_CHECK(apply<T>(ctx, a, vn, w));
    // Gram-Schmidt against every stored vector in order (modified: each
    // projection uses w after the previous subtraction); sc[j] = proj_j
    for (uint64_t j = 0; j < nv; ++j) {
      const T* vp = j ? V + (int64_t)(j - 1) * ldv : nullptr;
      SX_CHECK(launch_vec<T>(ctx, n, EgMgs<T>{w, vp, j ? W.sc + (j - 1) : nullptr, V + (int64_t)j * ldv, W.sc + j}));
    }
    // the last subtraction, then alpha = vn . w  (sc[nv])
    SX_CHECK(launch_vec<T>(ctx, n, EgMgs<T>{w, vn, W.sc + (nv - 1), vn, W.sc + nv}));
    // w -= alpha vn, ||w||^2 (sc[nv + 1])
    SX_CHECK(launch_vec<T>(ctx, n, EgAxpyNorm<T>{w, vn, W.sc + nv, W.sc + nv + 1}));
    std::vector<T> hv(nv + 2);
    SX_CHECK(W.read(hv.data(), (int)(nv + 2)));
    alpha.push_back(hv[nv]);
    const T bnext = std::sqrt(hv[nv + 1]);
    if (alpha.size() >= num) {
      SX_CHECK(tri_eig<T>(alpha, beta, num, te));
      if (te.vals.empty()) return err_panic("index out of bounds (no eigenvalue to test)");
      if (bnext < tol * std::fabs(te.vals[0])) { conv = true; break; }
    }
    ++it;
  }
  SX_CHECK(tri_eig<T>(alpha, beta, num, te));
  const int64_t cols = (int64_t)num;
  std::vector<T> resid(num, T(0));
  if (o.compute_eigenvectors) {
    // Ritz coefficients coef[j][k] = eigvecs[j][k] for j < min(#V, #eigvecs)
    const int nj = (int)std::min<uint64_t>(nv, te.vecs.size());
    std::vector<T> coef((size_t)std::max(nj, 1) * std::max<int64_t>(cols, 1), T(0));
    for (int j = 0; j < nj; ++j)
      for (int64_t k = 0; k < cols; ++k) {
        if ((size_t)k >= te.vecs[j].size()) return err_panic("index out of bounds in the eigenvector list");
        coef[(size_t)j * cols + k] = te.vecs[j][k];
      }
    for (int64_t k = 0; k < cols; ++k)
      if ((size_t)k >= te.vals.size()) return err_panic("index out of bounds in the eigenvalue list");
    T *dcoef = nullptr, *ritz = nullptr, *e = nullptr;
    SX_CHECK(W.alloc(&dcoef, (int64_t)coef.size()));
    SX_CHECK(W.alloc(&ritz, n * std::max<int64_t>(cols, 1)));
    SX_CHECK(W.alloc(&e, n));
    SX_CUDA(cudaMemcpyAsync(dcoef, coef.data(), coef.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    if (n > 0 && cols > 0) {
      k_ritz<T><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(V, n, ldv, nj, dcoef, (int)cols, ritz);
      ctx->launches++;
      SX_CUDA(cudaGetLastError());
    }
    for (int64_t k = 0; k < cols; ++k) {
      SX_CHECK(launch_vec<T>(ctx, n, EgColumn<T>{ritz, cols, k, e}));
      SX_CHECK(apply<T>(ctx, a, e, w));
      SX_CHECK(launch_vec<T>(ctx, n, EgResid<T>{w, e, te.vals[k], W.sc}));
      SX_CHECK(W.read(h, 1));
      resid[k] = std::sqrt(h[0]);
    }
    if (vecs_out) SX_CHECK(download<T>(ctx, ritz, n * cols, mem, vecs_out));
  } else {
    // Kaniel-Paige bound: beta_last |eigvecs[last][k]|
    for (uint64_t k = 0; k < num; ++k)
      if (k < te.vecs.size() && !beta.empty()) {
        if (k >= te.vecs.back().size()) return err_panic("index out of bounds in the eigenvector list");
        resid[k] = beta.back() * std::fabs(te.vecs.back()[k]);
      }
  }
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t k = 0; k < te.vals.size(); ++k) vals_out[k] = te.vals[k];
  for (uint64_t k = 0; k < num; ++k) resid_out[k] = resid[k];
  res->iterations = it;
  res->converged = conv ? 1 : 0;
  res->num_eigenvalues = te.vals.size();
  res->num_columns = num;
  return SX_OK;
}

bool sym_op(sx_op a) { return a && a->kind == SX_OP_SYM_CSR && a->sym_low; }

}  // namespace
}  // namespace sx

using namespace sx;

extern "C" {

void sx_power_options_default(sx_power_options* o) {
  if (!o) return;
  o->max_iter = 100;
  o->tol = 1e-8;
  o->normalize = 1;
}

void sx_lanczos_options_default(sx_lanczos_options* o) {
  if (!o) return;
  o->max_iter = 1000;
  o->max_subspace_size = 20;
  o->tol = 1e-8;
  o->num_eigenvalues = 1;
  o->compute_eigenvectors = 1;
}

int sx_power_iteration(sx_ctx ctx, sx_op a, const sx_power_options* opt, const void* x0, uint64_t x0_len, sx_mem mem,
                       void* eigenvalue, void* eigenvector, void* residual, sx_eigen_result* result) {
  if (!ctx || !eigenvalue || !residual || !result) return err_arg("null argument");
  if (!sym_op(a)) return err_arg("not a symmetric CSR operator");
  sx_power_options o;
  sx_power_options_default(&o);
  if (opt) o = *opt;
  if (x0 && x0_len != (uint64_t)a->nrows) return err_dim((uint64_t)a->nrows, x0_len);
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(a->dtype == SX_F64
               ? power_impl<double>(ctx, a, o, x0, mem, (double*)eigenvalue, eigenvector, (double*)residual, result)
               : power_impl<float>(ctx, a, o, x0, mem, (float*)eigenvalue, eigenvector, (float*)residual, result));
  return clear_error();
}

int sx_tridiag_eig(const double* alpha, const double* beta, uint64_t m, uint64_t beta_len, uint64_t num,
                   double* values, double* vectors, uint64_t* count) {
  if ((m > 0 && !alpha) || (beta_len > 0 && !beta) || !values || !vectors || !count)
    return err_arg("null argument");
  TriEig<double> te;
  SX_CHECK(tri_eig<double>(std::vector<double>(alpha, alpha + m), std::vector<double>(beta, beta + beta_len),
                           (size_t)num, te));
  *count = te.vals.size();
  for (size_t k = 0; k < te.vals.size(); ++k) values[k] = te.vals[k];
  for (size_t k = 0; k < te.vecs.size(); ++k)
    for (size_t i = 0; i < te.vecs[k].size(); ++i) vectors[k * m + i] = te.vecs[k][i];
  return clear_error();
}

int sx_lanczos(sx_ctx ctx, sx_op a, const sx_lanczos_options* opt, const void* v0, uint64_t v0_len, sx_mem mem,
               void* eigenvalues, void* eigenvectors, void* residuals, sx_eigen_result* result) {
  if (!ctx || !eigenvalues || !residuals || !result) return err_arg("null argument");
  if (!sym_op(a)) return err_arg("not a symmetric CSR operator");
  sx_lanczos_options o;
  sx_lanczos_options_default(&o);
  if (opt) o = *opt;
  if (v0 && v0_len != (uint64_t)a->nrows) return err_dim((uint64_t)a->nrows, v0_len);
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(a->dtype == SX_F64 ? lanczos_impl<double>(ctx, a, o, v0, mem, (double*)eigenvalues, eigenvectors,
                                                     (double*)residuals, result)
                              : lanczos_impl<float>(ctx, a, o, v0, mem, (float*)eigenvalues, eigenvectors,
                                                    (float*)residuals, result));
  return clear_error();
}

}  // extern "C"
