// scirs_sparse.hpp -- C++17 mirror of the scirs2-sparse iterative-solve API
// over the C ABI of include/scirs_sparse.h (header only).
//
// Names, argument meanings, option defaults and error variants follow the
// reference crate (scirs2-sparse, workspace 0.1.0-alpha.6):
//   CsrMatrix          csr.rs:15-498        (CsrMatrix::new -> CsrMatrix::create)
//   CsrArray           csr_array.rs:30-625  (CsrArray::new -> CsrArray::create)
//   LinearOperator     linalg/interface.rs:13-52, operators :55-223, :299-402
//   JacobiPreconditioner, IC0Preconditioner  linalg/preconditioners.rs:14-92, linalg/ic.rs:15-230
//   CGOptions / BiCGSTABOptions / GMRESOptions, cg / bicgstab / gmres,
//   IterationResult    linalg/iterative.rs:8-816
// Rust's SparseResult<T> becomes "returns T or throws SparseError"; the
// exception carries the SparseError variant, its payload and Display text.
// Every operation runs on the GPU through the library: an operator written
// by the user in C++ joins a device solve through a host callback.
#pragma once

#include <algorithm>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "scirs_sparse.h"

namespace scirs2_sparse {

// ------------------------------------------------------------------ errors
class SparseError : public std::runtime_error {
 public:
  SparseError(int code, std::string msg, uint64_t v0 = 0, uint64_t v1 = 0, uint64_t v2 = 0,
              uint64_t v3 = 0)
      : std::runtime_error(std::move(msg)), code(code), v0(v0), v1(v1), v2(v2), v3(v3) {}
  int code;
  uint64_t v0, v1, v2, v3;
  // the SparseError variant name (error.rs:9-74)
  std::string variant() const { return sx_status_string(code); }
};

namespace detail {
inline void check(int rc) {
  if (rc == SX_OK) return;
  sx_error_info e;
  sx_last_error(&e);
  throw SparseError(rc, e.message, e.v0, e.v1, e.v2, e.v3);
}
template <class F>
constexpr sx_dtype dtype_of() {
  static_assert(std::is_same<F, float>::value || std::is_same<F, double>::value,
                "F must be float or double");
  return std::is_same<F, double>::value ? SX_F64 : SX_F32;
}
}  // namespace detail

// One CUDA context (stream, scratch, graph caches) shared by default.
class Context {
 public:
  explicit Context(int device = 0) { detail::check(sx_ctx_create(device, &ctx_)); }
  ~Context() { sx_ctx_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  sx_ctx get() const { return ctx_; }
  static Context& global() {
    static Context c(0);
    return c;
  }

 private:
  sx_ctx ctx_ = nullptr;
};

// Owning handle of a device operator.
struct OpHandle {
  explicit OpHandle(sx_op h) : h(h) {}
  ~OpHandle() { sx_op_destroy(h); }
  OpHandle(const OpHandle&) = delete;
  OpHandle& operator=(const OpHandle&) = delete;
  sx_op h;
};

// ------------------------------------------------------- LinearOperator
template <class F>
class LinearOperator {
 public:
  virtual ~LinearOperator() = default;
  virtual std::pair<size_t, size_t> shape() const = 0;
  virtual std::vector<F> matvec(const std::vector<F>& x) const = 0;
  virtual std::vector<F> rmatvec(const std::vector<F>&) const {
    throw SparseError(SX_ERR_OPERATION_NOT_SUPPORTED,
                      "Operation not supported: adjoint not implemented for this operator");
  }
  virtual bool has_adjoint() const { return false; }
  // The device operator behind this LinearOperator; nullptr for a host-only
  // operator (it then joins device solves through a host callback).
  virtual sx_op device_op() const { return nullptr; }
};

// A LinearOperator backed by a device handle.
template <class F>
class DeviceOperator : public LinearOperator<F> {
 public:
  std::pair<size_t, size_t> shape() const override {
    uint64_t r = 0, c = 0;
    detail::check(sx_op_shape(op_->h, &r, &c));
    return {(size_t)r, (size_t)c};
  }
  std::vector<F> matvec(const std::vector<F>& x) const override {
    std::vector<F> y(shape().first);
    detail::check(sx_op_matvec(ctx_, op_->h, x.data(), x.size(), y.data(), SX_MEM_HOST));
    return y;
  }
  std::vector<F> rmatvec(const std::vector<F>& x) const override {
    std::vector<F> y(shape().second);
    detail::check(sx_op_rmatvec(ctx_, op_->h, x.data(), x.size(), y.data(), SX_MEM_HOST));
    return y;
  }
  bool has_adjoint() const override { return true; }
  sx_op device_op() const override { return op_->h; }
  sx_ctx context() const { return ctx_; }

 protected:
  DeviceOperator(sx_ctx ctx, sx_op h) : ctx_(ctx), op_(std::make_shared<OpHandle>(h)) {}
  sx_ctx ctx_;
  std::shared_ptr<OpHandle> op_;
};

// IdentityOperator, ScaledIdentityOperator, DiagonalOperator (interface.rs:55-175)
template <class F>
class IdentityOperator : public DeviceOperator<F> {
 public:
  explicit IdentityOperator(size_t n, Context& c = Context::global())
      : DeviceOperator<F>(c.get(), make(c.get(), n)) {}

 private:
  static sx_op make(sx_ctx ctx, size_t n) {
    sx_op h = nullptr;
    detail::check(sx_op_identity(ctx, detail::dtype_of<F>(), n, &h));
    return h;
  }
};

template <class F>
class ScaledIdentityOperator : public DeviceOperator<F> {
 public:
  ScaledIdentityOperator(size_t n, F scale, Context& c = Context::global())
      : DeviceOperator<F>(c.get(), make(c.get(), n, scale)) {}

 private:
  static sx_op make(sx_ctx ctx, size_t n, F scale) {
    sx_op h = nullptr;
    detail::check(sx_op_scaled_identity(ctx, detail::dtype_of<F>(), n, (double)scale, &h));
    return h;
  }
};

template <class F>
class DiagonalOperator : public DeviceOperator<F> {
 public:
  explicit DiagonalOperator(const std::vector<F>& diagonal, Context& c = Context::global())
      : DeviceOperator<F>(c.get(), make(c.get(), diagonal)), diagonal_(diagonal) {}
  const std::vector<F>& diagonal() const { return diagonal_; }

 private:
  static sx_op make(sx_ctx ctx, const std::vector<F>& d) {
    sx_op h = nullptr;
    detail::check(sx_op_diagonal(ctx, detail::dtype_of<F>(), d.data(), d.size(), &h));
    return h;
  }
  std::vector<F> diagonal_;
};

// ZeroOperator (interface.rs:177-222)
template <class F>
class ZeroOperator : public DeviceOperator<F> {
 public:
  ZeroOperator(size_t rows, size_t cols, Context& c = Context::global())
      : DeviceOperator<F>(c.get(), make(c.get(), rows, cols)) {}

 private:
  static sx_op make(sx_ctx ctx, size_t rows, size_t cols) {
    sx_op h = nullptr;
    detail::check(sx_op_zero(ctx, detail::dtype_of<F>(), rows, cols, &h));
    return h;
  }
};

// SumOperator (A + B) and ProductOperator (A B) (interface.rs:299-402).  The
// reference boxes its operands; here the composite keeps shared references
// to the two device operators, so they live as long as it does.
template <class F>
class SumOperator : public DeviceOperator<F> {
 public:
  static SumOperator create(std::shared_ptr<DeviceOperator<F>> a, std::shared_ptr<DeviceOperator<F>> b) {
    sx_op h = nullptr;
    detail::check(sx_op_sum(a->context(), a->device_op(), b->device_op(), &h));
    return SumOperator(a->context(), h, a, b);
  }
  bool has_adjoint() const override { return a_->has_adjoint() && b_->has_adjoint(); }

 private:
  SumOperator(sx_ctx ctx, sx_op h, std::shared_ptr<DeviceOperator<F>> a, std::shared_ptr<DeviceOperator<F>> b)
      : DeviceOperator<F>(ctx, h), a_(std::move(a)), b_(std::move(b)) {}
  std::shared_ptr<DeviceOperator<F>> a_, b_;
};

template <class F>
class ProductOperator : public DeviceOperator<F> {
 public:
  static ProductOperator create(std::shared_ptr<DeviceOperator<F>> a, std::shared_ptr<DeviceOperator<F>> b) {
    sx_op h = nullptr;
    detail::check(sx_op_product(a->context(), a->device_op(), b->device_op(), &h));
    return ProductOperator(a->context(), h, a, b);
  }
  bool has_adjoint() const override { return a_->has_adjoint() && b_->has_adjoint(); }

 private:
  ProductOperator(sx_ctx ctx, sx_op h, std::shared_ptr<DeviceOperator<F>> a,
                  std::shared_ptr<DeviceOperator<F>> b)
      : DeviceOperator<F>(ctx, h), a_(std::move(a)), b_(std::move(b)) {}
  std::shared_ptr<DeviceOperator<F>> a_, b_;
};

// ------------------------------------------------------------------ CSR
template <class F>
class CsrBase : public DeviceOperator<F> {
 public:
  size_t rows() const { return this->shape().first; }
  size_t cols() const { return this->shape().second; }
  size_t nnz() const {
    uint64_t r = 0, c = 0, z = 0;
    int s = 0;
    detail::check(sx_csr_info(this->op_->h, &r, &c, &z, &s));
    return (size_t)z;
  }
  // get(i, j): first stored entry, zero when absent or out of range (csr.rs:33-48)
  F get(size_t i, size_t j) const {
    F v = F(0);
    detail::check(sx_csr_get(this->ctx_, this->op_->h, i, j, &v));
    return v;
  }
  // the public arrays (csr.rs:20-25)
  std::vector<size_t> indptr() const { return arrays().first.first; }
  std::vector<size_t> indices() const { return arrays().first.second; }
  std::vector<F> data() const { return arrays().second; }
  std::vector<std::vector<F>> to_dense() const {
    auto a = arrays();
    std::vector<std::vector<F>> d(rows(), std::vector<F>(cols(), F(0)));
    for (size_t r = 0; r < rows(); ++r)
      for (size_t k = a.first.first[r]; k < a.first.first[r + 1]; ++k) d[r][a.first.second[k]] = a.second[k];
    return d;
  }

 protected:
  using DeviceOperator<F>::DeviceOperator;
  std::pair<std::pair<std::vector<size_t>, std::vector<size_t>>, std::vector<F>> arrays() const {
    std::vector<uint64_t> ip(rows() + 1), ix(nnz());
    std::vector<F> d(nnz());
    detail::check(sx_csr_download(this->ctx_, this->op_->h, ip.data(), ix.data(), d.data()));
    return {{std::vector<size_t>(ip.begin(), ip.end()), std::vector<size_t>(ix.begin(), ix.end())}, d};
  }
  static std::vector<uint64_t> u64(const std::vector<size_t>& v) {
    return std::vector<uint64_t>(v.begin(), v.end());
  }
};

template <class F>
class CsrMatrix : public CsrBase<F> {
 public:
  // CsrMatrix::new(data, row_indices, col_indices, shape) (csr.rs:92-160)
  static CsrMatrix create(const std::vector<F>& data, const std::vector<size_t>& rows,
                          const std::vector<size_t>& cols, std::pair<size_t, size_t> shape,
                          Context& c = Context::global()) {
    if (data.size() != rows.size() || data.size() != cols.size()) {
      const size_t found = std::min(rows.size(), cols.size());
      throw SparseError(SX_ERR_DIMENSION_MISMATCH,
                        "Dimension mismatch: expected " + std::to_string(data.size()) + ", found " +
                            std::to_string(found),
                        data.size(), found);
    }
    auto r = CsrBase<F>::u64(rows), k = CsrBase<F>::u64(cols);
    sx_op h = nullptr;
    detail::check(sx_csr_from_triplets(c.get(), detail::dtype_of<F>(), SX_API_CSR_MATRIX, r.data(),
                                       k.data(), data.data(), data.size(), shape.first, shape.second,
                                       0, &h));
    return CsrMatrix(c.get(), h);
  }
  // CsrMatrix::from_raw_csr(data, indptr, indices, shape) (csr.rs:174-227)
  static CsrMatrix from_raw_csr(const std::vector<F>& data, const std::vector<size_t>& indptr,
                                const std::vector<size_t>& indices, std::pair<size_t, size_t> shape,
                                Context& c = Context::global()) {
    if (indptr.size() == shape.first + 1 && data.size() != indices.size())
      throw SparseError(SX_ERR_DIMENSION_MISMATCH,
                        "Dimension mismatch: expected " + std::to_string(data.size()) + ", found " +
                            std::to_string(indices.size()),
                        data.size(), indices.size());
    auto p = CsrBase<F>::u64(indptr), k = CsrBase<F>::u64(indices);
    sx_op h = nullptr;
    detail::check(sx_csr_from_raw(c.get(), detail::dtype_of<F>(), SX_API_CSR_MATRIX, p.data(),
                                  p.size(), k.data(), data.data(), std::min(data.size(), k.size()),
                                  shape.first, shape.second, &h));
    return CsrMatrix(c.get(), h);
  }
  CsrMatrix transpose() const {
    sx_op h = nullptr;
    detail::check(sx_csr_transpose(this->ctx_, this->op_->h, &h));
    return CsrMatrix(this->ctx_, h);
  }
  // CsrMatrix<f64>::dot (csr.rs:479-497)
  std::vector<F> dot(const std::vector<F>& x) const { return this->matvec(x); }
  // takes ownership of a CSR handle made by another call of the library
  static CsrMatrix adopt(sx_ctx ctx, sx_op h) { return CsrMatrix(ctx, h); }

 private:
  CsrMatrix(sx_ctx ctx, sx_op h) : CsrBase<F>(ctx, h) {}
};

template <class F>
class CsrArray : public CsrBase<F> {
 public:
  // CsrArray::new(data, indices, indptr, shape) (csr_array.rs:77-136)
  static CsrArray create(const std::vector<F>& data, const std::vector<size_t>& indices,
                         const std::vector<size_t>& indptr, std::pair<size_t, size_t> shape,
                         Context& c = Context::global()) {
    if (data.size() != indices.size())
      throw SparseError(SX_ERR_INCONSISTENT_DATA,
                        "Inconsistent data: data and indices must have the same length");
    auto p = CsrBase<F>::u64(indptr), k = CsrBase<F>::u64(indices);
    sx_op h = nullptr;
    detail::check(sx_csr_from_raw(c.get(), detail::dtype_of<F>(), SX_API_CSR_ARRAY, p.data(), p.size(),
                                  k.data(), data.data(), data.size(), shape.first, shape.second, &h));
    return CsrArray(c.get(), h);
  }
  // CsrArray::from_triplets(rows, cols, data, shape, sorted) (csr_array.rs:152-219)
  static CsrArray from_triplets(const std::vector<size_t>& rows, const std::vector<size_t>& cols,
                                const std::vector<F>& data, std::pair<size_t, size_t> shape, bool sorted,
                                Context& c = Context::global()) {
    if (rows.size() != cols.size() || rows.size() != data.size())
      throw SparseError(SX_ERR_INCONSISTENT_DATA,
                        "Inconsistent data: rows, cols, and data must have the same length");
    auto r = CsrBase<F>::u64(rows), k = CsrBase<F>::u64(cols);
    sx_op h = nullptr;
    detail::check(sx_csr_from_triplets(c.get(), detail::dtype_of<F>(), SX_API_CSR_ARRAY, r.data(),
                                       k.data(), data.data(), data.size(), shape.first, shape.second,
                                       sorted ? 1 : 0, &h));
    return CsrArray(c.get(), h);
  }
  // SparseArray::dot_vector (csr_array.rs:569-593)
  std::vector<F> dot_vector(const std::vector<F>& x) const { return this->matvec(x); }
  CsrArray transpose() const {
    sx_op h = nullptr;
    detail::check(sx_csr_transpose(this->ctx_, this->op_->h, &h));
    return CsrArray(this->ctx_, h);
  }
  bool has_sorted_indices() const {
    uint64_t r = 0, c = 0, z = 0;
    int s = 0;
    detail::check(sx_csr_info(this->op_->h, &r, &c, &z, &s));
    return s != 0;
  }

 private:
  CsrArray(sx_ctx ctx, sx_op h) : CsrBase<F>(ctx, h) {}
};

// -------------------------------------------------------- preconditioners
// ------------------------------------------- SymCsrMatrix (sym_csr.rs:24-337)
// The lower triangle is stored; matvec / get apply the full symmetric matrix.
template <class F>
class SymCsrMatrix : public DeviceOperator<F> {
 public:
  // SymCsrMatrix::new(data, indptr, indices, shape) (sym_csr.rs:64-134)
  static SymCsrMatrix create(const std::vector<F>& data, const std::vector<size_t>& indptr,
                             const std::vector<size_t>& indices, std::pair<size_t, size_t> shape,
                             Context& c = Context::global()) {
    std::vector<uint64_t> p(indptr.begin(), indptr.end()), k(indices.begin(), indices.end());
    sx_op h = nullptr;
    detail::check(sx_sym_csr_new(c.get(), detail::dtype_of<F>(), data.data(), data.size(), p.data(),
                                 p.size(), k.data(), k.size(), shape.first, shape.second, &h));
    return SymCsrMatrix(c.get(), h);
  }
  // SymCsrMatrix::from_csr (sym_csr.rs:149-189)
  static SymCsrMatrix from_csr(const CsrMatrix<F>& m) {
    sx_op h = nullptr;
    detail::check(sx_sym_csr_from_csr(m.context(), m.device_op(), &h));
    return SymCsrMatrix(m.context(), h);
  }
  size_t nnz_stored() const { return (size_t)info().first; }
  size_t nnz() const { return (size_t)info().second; }
  F get(size_t i, size_t j) const {
    F v = F(0);
    detail::check(sx_csr_get(this->ctx_, this->op_->h, i, j, &v));
    return v;
  }
  std::vector<size_t> indptr() const { return arrays().first.first; }
  std::vector<size_t> indices() const { return arrays().first.second; }
  std::vector<F> data() const { return arrays().second; }
  // SymCsrMatrix::to_csr (sym_csr.rs:305-337)
  CsrMatrix<F> to_csr() const {
    sx_op h = nullptr;
    detail::check(sx_sym_csr_to_csr(this->ctx_, this->op_->h, &h));
    return CsrMatrix<F>::adopt(this->ctx_, h);
  }
  // SymCsrMatrix::to_dense (sym_csr.rs:344-366)
  std::vector<std::vector<F>> to_dense() const {
    auto a = arrays();
    const size_t n = this->shape().first;
    std::vector<std::vector<F>> d(n, std::vector<F>(n, F(0)));
    for (size_t r = 0; r < n; ++r)
      for (size_t k = a.first.first[r]; k < a.first.first[r + 1]; ++k) d[r][a.first.second[k]] = a.second[k];
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < i; ++j) d[j][i] = d[i][j];
    return d;
  }

 private:
  SymCsrMatrix(sx_ctx ctx, sx_op h) : DeviceOperator<F>(ctx, h) {}
  std::pair<uint64_t, uint64_t> info() const {
    uint64_t a = 0, b = 0;
    detail::check(sx_sym_csr_info(this->ctx_, this->op_->h, &a, &b));
    return {a, b};
  }
  std::pair<std::pair<std::vector<size_t>, std::vector<size_t>>, std::vector<F>> arrays() const {
    std::vector<uint64_t> ip(this->shape().first + 1), ix(nnz_stored());
    std::vector<F> d(nnz_stored());
    detail::check(sx_sym_csr_download(this->ctx_, this->op_->h, ip.data(), ix.data(), d.data()));
    return {{std::vector<size_t>(ip.begin(), ip.end()), std::vector<size_t>(ix.begin(), ix.end())}, d};
  }
};

// sym_ops.rs:56-90, :179-233, :271-283, :317-335
template <class F>
std::vector<F> sym_csr_matvec(const SymCsrMatrix<F>& m, const std::vector<F>& x) {
  return m.matvec(x);
}
template <class F>
void sym_csr_rank1_update(SymCsrMatrix<F>& m, const std::vector<F>& x, F alpha) {
  detail::check(sx_sym_csr_rank1_update(m.context(), m.device_op(), x.data(), x.size(), (double)alpha,
                                        SX_MEM_HOST));
}
template <class F>
F sym_csr_quadratic_form(const SymCsrMatrix<F>& m, const std::vector<F>& x) {
  F v = F(0);
  detail::check(sx_sym_csr_quadratic_form(m.context(), m.device_op(), x.data(), x.size(), SX_MEM_HOST, &v));
  return v;
}
template <class F>
F sym_csr_trace(const SymCsrMatrix<F>& m) {
  F v = F(0);
  detail::check(sx_sym_csr_trace(m.context(), m.device_op(), &v));
  return v;
}

template <class F>
class JacobiPreconditioner : public DeviceOperator<F> {
 public:
  // JacobiPreconditioner::new(&matrix) (preconditioners.rs:21-44)
  static JacobiPreconditioner create(const CsrBase<F>& matrix) {
    sx_op h = nullptr;
    detail::check(sx_precond_jacobi(matrix.context(), matrix.device_op(), &h));
    return JacobiPreconditioner(matrix.context(), h);
  }
  // JacobiPreconditioner::from_diagonal (preconditioners.rs:47-62)
  static JacobiPreconditioner from_diagonal(const std::vector<F>& diagonal,
                                            Context& c = Context::global()) {
    sx_op h = nullptr;
    detail::check(sx_precond_jacobi_from_diagonal(c.get(), detail::dtype_of<F>(), diagonal.data(),
                                                  diagonal.size(), &h));
    return JacobiPreconditioner(c.get(), h);
  }

 private:
  JacobiPreconditioner(sx_ctx ctx, sx_op h) : DeviceOperator<F>(ctx, h) {}
};

template <class F>
class IC0Preconditioner : public DeviceOperator<F> {
 public:
  // IC0Preconditioner::new(&matrix) (ic.rs:22-135); textbook = standard IC(0)
  static IC0Preconditioner create(const CsrBase<F>& matrix, bool textbook = false) {
    sx_op h = nullptr;
    detail::check(sx_precond_ic0(matrix.context(), matrix.device_op(),
                                 textbook ? SX_IC0_TEXTBOOK : SX_IC0_REFERENCE, &h));
    return IC0Preconditioner(matrix.context(), h);
  }

 private:
  IC0Preconditioner(sx_ctx ctx, sx_op h) : DeviceOperator<F>(ctx, h) {}
};

// ------------------------------------------------------------- solvers
template <class F>
struct IterationResult {  // iterative.rs:8-14
  std::vector<F> x;
  size_t iterations = 0;
  F residual_norm = F(0);
  bool converged = false;
  std::string message;
};

template <class F>
using OperatorPtr = std::shared_ptr<LinearOperator<F>>;

template <class F>
struct CGOptions {  // iterative.rs:17-35
  size_t max_iter = 1000;
  F rtol = F(1e-8);
  F atol = F(1e-12);
  std::vector<F> x0;  // empty = zeros (None)
  OperatorPtr<F> preconditioner;
};
template <class F>
struct BiCGSTABOptions {  // iterative.rs:348-368
  size_t max_iter = 1000;
  F rtol = F(1e-8);
  F atol = F(1e-12);
  std::vector<F> x0;
  OperatorPtr<F> left_preconditioner;
  OperatorPtr<F> right_preconditioner;
};
template <class F>
struct GMRESOptions {  // iterative.rs:614-634
  size_t max_iter = 1000;
  size_t restart = 30;
  F rtol = F(1e-8);
  F atol = F(1e-12);
  std::vector<F> x0;
  OperatorPtr<F> preconditioner;
};

template <class F>
struct BiCGOptions {  // iterative.rs:164-185; also CGSOptions (cgs.rs:8) and QMROptions (qmr.rs:18-38)
  size_t max_iter = 1000;
  F rtol = F(1e-8);
  F atol = F(1e-12);
  std::vector<F> x0;
  OperatorPtr<F> left_preconditioner;
  OperatorPtr<F> right_preconditioner;
};
template <class F>
using CGSOptions = BiCGOptions<F>;
template <class F>
using QMROptions = BiCGOptions<F>;
template <class F>
struct MINRESOptions {  // minres.rs:17-35
  size_t max_iter = 1000;
  F rtol = F(1e-8);
  F atol = F(1e-12);
  std::vector<F> x0;
  OperatorPtr<F> preconditioner;
};
template <class F>
struct LGMRESOptions {  // lgmres.rs:10-38
  size_t max_iter = 500;
  F rtol = F(1e-8);
  F atol = F(1e-8);
  size_t inner_m = 30;
  size_t outer_k = 3;
  std::vector<F> x0;
  OperatorPtr<F> preconditioner;
};

namespace detail {
// A device handle for any operator: its own, or a host callback for a
// user-defined C++ LinearOperator (staged copies; the loop stays on the GPU).
template <class F>
struct OpRef {
  sx_op h = nullptr;
  std::unique_ptr<OpHandle> owned;
};
template <class F>
int host_matvec_thunk(void* user, const void* x, void* y, uint64_t n) {
  try {
    auto* op = static_cast<const LinearOperator<F>*>(user);
    std::vector<F> xv((const F*)x, (const F*)x + n);
    std::vector<F> yv = op->matvec(xv);
    std::copy(yv.begin(), yv.end(), (F*)y);
    return 0;
  } catch (...) {
    return 1;
  }
}
template <class F>
OpRef<F> device_ref(const LinearOperator<F>* op, sx_ctx ctx) {
  OpRef<F> r;
  if (!op) return r;
  r.h = op->device_op();
  if (!r.h) {
    auto s = op->shape();
    sx_op h = nullptr;
    check(sx_op_host(ctx, dtype_of<F>(), s.first, s.second, &host_matvec_thunk<F>,
                     const_cast<LinearOperator<F>*>(op), &h));
    r.owned.reset(new OpHandle(h));
    r.h = h;
  }
  return r;
}
template <class F>
IterationResult<F> result(std::vector<F>&& x, const sx_iter_result& r) {
  IterationResult<F> out;
  out.x = std::move(x);
  out.iterations = (size_t)r.iterations;
  out.residual_norm = (F)r.residual_norm;
  out.converged = r.converged != 0;
  char buf[512];
  check(sx_iter_message(&r, dtype_of<F>(), buf, sizeof(buf)));
  out.message = buf;
  return out;
}
template <class F>
IterationResult<F> bicg_like(int (*fn)(sx_ctx, sx_op, const void*, uint64_t, const sx_bicg_options*, void*,
                                       sx_mem, sx_iter_result*),
                             const LinearOperator<F>& a, const std::vector<F>& b, const BiCGOptions<F>& options,
                             Context& c) {
  auto A = device_ref(&a, c.get());
  auto M1 = device_ref(options.left_preconditioner.get(), c.get());
  auto M2 = device_ref(options.right_preconditioner.get(), c.get());
  sx_bicg_options o;
  sx_bicg_options_default(&o);
  o.max_iter = options.max_iter;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.left_preconditioner = M1.h;
  o.right_preconditioner = M2.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  check(fn(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return result(std::move(x), r);
}
}  // namespace detail

// cg(a, b, options) (iterative.rs:40-162)
template <class F>
IterationResult<F> cg(const LinearOperator<F>& a, const std::vector<F>& b, CGOptions<F> options,
                      Context& c = Context::global()) {
  auto A = detail::device_ref(&a, c.get());
  auto M = detail::device_ref(options.preconditioner.get(), c.get());
  sx_cg_options o;
  sx_cg_options_default(&o);
  o.max_iter = options.max_iter;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.preconditioner = M.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  detail::check(sx_cg(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return detail::result(std::move(x), r);
}

// bicgstab(a, b, options) (iterative.rs:377-611)
template <class F>
IterationResult<F> bicgstab(const LinearOperator<F>& a, const std::vector<F>& b,
                            BiCGSTABOptions<F> options, Context& c = Context::global()) {
  auto A = detail::device_ref(&a, c.get());
  auto M1 = detail::device_ref(options.left_preconditioner.get(), c.get());
  auto M2 = detail::device_ref(options.right_preconditioner.get(), c.get());
  sx_bicgstab_options o;
  sx_bicgstab_options_default(&o);
  o.max_iter = options.max_iter;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.left_preconditioner = M1.h;
  o.right_preconditioner = M2.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  detail::check(sx_bicgstab(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return detail::result(std::move(x), r);
}

// gmres(a, b, options) (iterative.rs:641-816)
template <class F>
IterationResult<F> gmres(const LinearOperator<F>& a, const std::vector<F>& b, GMRESOptions<F> options,
                         Context& c = Context::global()) {
  auto A = detail::device_ref(&a, c.get());
  auto M = detail::device_ref(options.preconditioner.get(), c.get());
  sx_gmres_options o;
  sx_gmres_options_default(&o);
  o.max_iter = options.max_iter;
  o.restart = options.restart;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.preconditioner = M.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  detail::check(sx_gmres(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return detail::result(std::move(x), r);
}

// bicg (iterative.rs:189-345), cgs (cgs.rs:15-193), qmr (qmr.rs:44-259)
template <class F>
IterationResult<F> bicg(const LinearOperator<F>& a, const std::vector<F>& b, BiCGOptions<F> options,
                        Context& c = Context::global()) {
  return detail::bicg_like(&sx_bicg, a, b, options, c);
}
template <class F>
IterationResult<F> cgs(const LinearOperator<F>& a, const std::vector<F>& b, CGSOptions<F> options,
                       Context& c = Context::global()) {
  return detail::bicg_like(&sx_cgs, a, b, options, c);
}
template <class F>
IterationResult<F> qmr(const LinearOperator<F>& a, const std::vector<F>& b, QMROptions<F> options,
                       Context& c = Context::global()) {
  return detail::bicg_like(&sx_qmr, a, b, options, c);
}

// minres (minres.rs:66-257)
template <class F>
IterationResult<F> minres(const LinearOperator<F>& a, const std::vector<F>& b, MINRESOptions<F> options,
                          Context& c = Context::global()) {
  auto A = detail::device_ref(&a, c.get());
  auto M = detail::device_ref(options.preconditioner.get(), c.get());
  sx_minres_options o;
  sx_minres_options_default(&o);
  o.max_iter = options.max_iter;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.preconditioner = M.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  detail::check(sx_minres(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return detail::result(std::move(x), r);
}

// lgmres (lgmres.rs:58-327); LGMRESResult carries no message
template <class F>
IterationResult<F> lgmres(const LinearOperator<F>& a, const std::vector<F>& b, LGMRESOptions<F> options,
                          Context& c = Context::global()) {
  auto A = detail::device_ref(&a, c.get());
  auto M = detail::device_ref(options.preconditioner.get(), c.get());
  sx_lgmres_options o;
  sx_lgmres_options_default(&o);
  o.max_iter = options.max_iter;
  o.rtol = (double)options.rtol;
  o.atol = (double)options.atol;
  o.inner_m = options.inner_m;
  o.outer_k = options.outer_k;
  o.x0 = options.x0.empty() ? nullptr : options.x0.data();
  o.preconditioner = M.h;
  std::vector<F> x(a.shape().first);
  sx_iter_result r;
  detail::check(sx_lgmres(c.get(), A.h, b.data(), b.size(), &o, x.data(), SX_MEM_HOST, &r));
  return detail::result(std::move(x), r);
}

// ---------------------------------------------------------- eigenpairs
// EigenResult (eigen.rs:64-78); eigenvectors is n x k row-major (column k =
// pair k), empty when not computed.
template <class F>
struct EigenResult {
  std::vector<F> eigenvalues;
  std::vector<F> eigenvectors;
  std::size_t rows = 0, cols = 0;
  std::size_t iterations = 0;
  std::vector<F> residuals;
  bool converged = false;
};
struct PowerIterationOptions {  // eigen.rs:16-34
  std::size_t max_iter = 100;
  double tol = 1e-8;
  bool normalize = true;
};
struct LanczosOptions {  // eigen.rs:37-61
  std::size_t max_iter = 1000;
  std::size_t max_subspace_size = 20;
  double tol = 1e-8;
  std::size_t num_eigenvalues = 1;
  bool compute_eigenvectors = true;
};

// power_iteration (eigen.rs:124-293); an empty initial guess means e_0
template <class F>
EigenResult<F> power_iteration(const SymCsrMatrix<F>& m, const PowerIterationOptions& options,
                               const std::vector<F>& initial_guess = {}) {
  const std::size_t n = m.shape().first;
  sx_power_options o{options.max_iter, options.tol, options.normalize ? 1 : 0};
  EigenResult<F> r;
  r.eigenvalues.assign(1, F(0));
  r.residuals.assign(1, F(0));
  r.eigenvectors.assign(n, F(0));
  sx_eigen_result e;
  detail::check(sx_power_iteration(m.context(), m.device_op(), &o,
                                   initial_guess.empty() ? nullptr : initial_guess.data(), initial_guess.size(),
                                   SX_MEM_HOST, r.eigenvalues.data(), r.eigenvectors.data(), r.residuals.data(), &e));
  r.rows = n;
  r.cols = 1;
  r.iterations = e.iterations;
  r.converged = e.converged != 0;
  return r;
}

// lanczos (eigen.rs:295-494)
template <class F>
EigenResult<F> lanczos(const SymCsrMatrix<F>& m, const LanczosOptions& options,
                       const std::vector<F>& initial_guess = {}) {
  const std::size_t n = m.shape().first;
  const std::size_t k = std::max<std::size_t>(
      std::min(options.num_eigenvalues, std::min(options.max_subspace_size, n)), 1);
  sx_lanczos_options o{options.max_iter, options.max_subspace_size, options.tol, options.num_eigenvalues,
                       options.compute_eigenvectors ? 1 : 0};
  EigenResult<F> r;
  r.eigenvalues.assign(k, F(0));
  r.residuals.assign(k, F(0));
  if (options.compute_eigenvectors) r.eigenvectors.assign(n * k, F(0));
  sx_eigen_result e;
  detail::check(sx_lanczos(m.context(), m.device_op(), &o, initial_guess.empty() ? nullptr : initial_guess.data(),
                           initial_guess.size(), SX_MEM_HOST, r.eigenvalues.data(),
                           options.compute_eigenvectors ? r.eigenvectors.data() : nullptr, r.residuals.data(), &e));
  r.eigenvalues.resize(e.num_eigenvalues);
  r.residuals.resize(e.num_columns);
  if (options.compute_eigenvectors) r.eigenvectors.resize(n * e.num_columns);
  r.rows = n;
  r.cols = options.compute_eigenvectors ? e.num_columns : 0;
  r.iterations = e.iterations;
  r.converged = e.converged != 0;
  return r;
}

}  // namespace scirs2_sparse
