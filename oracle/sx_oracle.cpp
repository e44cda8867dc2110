// CPU oracle for the scirs2-sparse iterative-solve path -- TEST INFRASTRUCTURE.
//
// A restatement, in C++17, of the reference functions listed beside each
// routine (paths relative to the reference workspace).  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library,
// and only as the checker or the timed CPU baseline: the product never does.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off).  The flag matters: Rust
// evaluates `sum += a * b` as a rounded product followed by a rounded add.
//
// Parity pins: tests/test_oracle_golden.py replays the reference's own unit
// and integration tests against this file (csr.rs, csr_array.rs, lib.rs,
// iterative.rs, preconditioners.rs, ic.rs tests and tests/*.rs).  gmres has
// no test in the reference crate: its parity is pinned only by this
// restatement.

#include "sx_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------- worker pool
// Row-parallel SpMV and elementwise vector loops may run on several host
// threads (or_set_threads; one by default, like the reference).  Each row's
// sum and each element's update keep their own arithmetic, so the results
// are bit-identical to the single-threaded loops.  Reductions (dot, norm2)
// always stay strict left folds on the calling thread.
class Pool {
 public:
  ~Pool() { resize(1); }
  int size() const { return nthreads_; }
  void resize(int nt) {
    if (nt < 1) nt = 1;
    if (nt == nthreads_) return;
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
    workers_.clear();
    stop_ = false;
    nthreads_ = nt;
    // a worker starts from the generation current now, so a job dispatched
    // before it first takes the lock is still seen as new
    const uint64_t g0 = gen_;
    for (int w = 1; w < nt; ++w) workers_.emplace_back([this, w, g0]() { loop(w, g0); });
  }
  // fn(lo, hi) over [0, n) in nthreads contiguous pieces
  void run(int64_t n, const std::function<void(int64_t, int64_t)>& fn) {
    if (nthreads_ == 1 || n < 4096) {
      fn(0, n);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &fn;
      n_ = n;
      pending_ = nthreads_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    piece(0, fn);
    std::unique_lock<std::mutex> g(m_);
    done_.wait(g, [this]() { return pending_ == 0; });
    job_ = nullptr;
  }

 private:
  void piece(int w, const std::function<void(int64_t, int64_t)>& fn) {
    const int64_t chunk = (n_ + nthreads_ - 1) / nthreads_;
    const int64_t lo = std::min<int64_t>(n_, w * chunk), hi = std::min<int64_t>(n_, lo + chunk);
    if (lo < hi) fn(lo, hi);
  }
  void loop(int w, uint64_t seen) {
    for (;;) {
      const std::function<void(int64_t, int64_t)>* job;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&]() { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        job = job_;
      }
      piece(w, *job);
      {
        std::lock_guard<std::mutex> g(m_);
        if (--pending_ == 0) done_.notify_one();
      }
    }
  }
  int nthreads_ = 1;
  std::vector<std::thread> workers_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  uint64_t gen_ = 0;
  bool stop_ = false;
  const std::function<void(int64_t, int64_t)>* job_ = nullptr;
  int64_t n_ = 0;
  int pending_ = 0;
};

Pool& pool() {
  static Pool p;
  return p;
}

template <class Fn>
void par_for(int64_t n, Fn fn) {
  pool().run(n, std::function<void(int64_t, int64_t)>(fn));
}

enum ErrCode {
  E_OK = 0,
  E_COMPUTATION = 1,
  E_DIMENSION_MISMATCH = 2,
  E_INDEX_OUT_OF_BOUNDS = 3,
  E_INVALID_AXIS = 4,
  E_INVALID_SLICE = 5,
  E_INCONSISTENT_DATA = 6,
  E_NOT_IMPLEMENTED = 7,
  E_SINGULAR = 8,
  E_VALUE = 9,
  E_CONVERSION = 10,
  E_NOT_SUPPORTED = 11,
  E_SHAPE_MISMATCH = 12,
  E_SOLVER_FAILURE = 13,
  E_INDEX_CAST_OVERFLOW = 14,
};

enum Msg {
  M_CONVERGED = 0,
  M_MAX_ITER = 1,
  M_NOT_PD = 2,
  M_CONVERGED_INITIAL = 3,
  M_BD_RHO = 4,
  M_BD_RHAT_V = 5,
  M_BD_ALPHA = 6,
  M_BD_TT = 7,
  M_BD_OMEGA = 8,
  M_BICG_PQ = 9,
  M_BICG_RHO = 10,
  M_CGS_RHO = 11,
  M_CGS_SIGMA = 12,
  M_QMR_INITIAL = 13,
  M_QMR_RHO = 14,
  M_QMR_PQ = 15,
  M_QMR_CONVERGED = 16,
  M_QMR_OMEGA = 17,
  M_QMR_MAX_ITER = 18,
  M_ZERO_RHS = 19,
  M_ZERO_RESIDUAL = 20,
};

int set_err(or_err* e, int code, const std::string& msg, uint64_t v0 = 0, uint64_t v1 = 0,
            uint64_t v2 = 0, uint64_t v3 = 0) {
  if (e) {
    e->code = code;
    e->v0 = v0; e->v1 = v1; e->v2 = v2; e->v3 = v3;
    std::snprintf(e->msg, sizeof(e->msg), "%s", msg.c_str());
  }
  return code;
}
int ok(or_err* e) {
  if (e) { e->code = 0; e->msg[0] = 0; }
  return 0;
}
std::string dim_msg(uint64_t expected, uint64_t found) {
  return "Dimension mismatch: expected " + std::to_string(expected) + ", found " +
         std::to_string(found);
}
std::string value_msg(const std::string& s) { return "Value error: " + s; }
std::string incons_msg(const std::string& s) { return "Inconsistent data: " + s; }

// ------------------------------------------------------------------ CSR
// CsrMatrix::new, scirs2-sparse/src/csr.rs:92-160.  The caller's single nnz
// argument already implies equal lengths of data/rows/cols.
template <class T>
int csr_matrix_new(const T* data, const uint64_t* rows, const uint64_t* cols, uint64_t nnz,
                   uint64_t nrows, uint64_t ncols, uint64_t* indptr, uint64_t* indices, T* out,
                   or_err* err) {
  for (uint64_t k = 0; k < nnz; ++k)
    if (rows[k] >= nrows) return set_err(err, E_VALUE, value_msg("Row index out of bounds"));
  for (uint64_t k = 0; k < nnz; ++k)
    if (cols[k] >= ncols) return set_err(err, E_VALUE, value_msg("Column index out of bounds"));
  // stable sort by (row, col): duplicates are kept in input order (csr.rs:129)
  std::vector<uint64_t> perm(nnz);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](uint64_t a, uint64_t b) {
    if (rows[a] != rows[b]) return rows[a] < rows[b];
    return cols[a] < cols[b];
  });
  for (uint64_t i = 0; i <= nrows; ++i) indptr[i] = 0;
  for (uint64_t k = 0; k < nnz; ++k) indptr[rows[k] + 1] += 1;
  for (uint64_t i = 1; i <= nrows; ++i) indptr[i] += indptr[i - 1];
  for (uint64_t k = 0; k < nnz; ++k) {
    indices[k] = cols[perm[k]];
    out[k] = data[perm[k]];
  }
  return ok(err);
}

// CsrMatrix::from_raw_csr validation, csr.rs:174-227 (the arrays are kept
// as given).
int csr_matrix_from_raw_check(const uint64_t* indptr, uint64_t indptr_len, const uint64_t* indices,
                              uint64_t indices_len, uint64_t data_len, uint64_t nrows,
                              uint64_t ncols, or_err* err) {
  if (indptr_len != nrows + 1)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(nrows + 1, indptr_len), nrows + 1,
                   indptr_len);
  if (data_len != indices_len)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(data_len, indices_len), data_len,
                   indices_len);
  for (uint64_t i = 1; i < indptr_len; ++i)
    if (indptr[i] < indptr[i - 1])
      return set_err(err, E_VALUE,
                     value_msg("Row pointer array must be monotonically increasing"));
  if (indptr[nrows] != data_len)
    return set_err(err, E_VALUE, value_msg("Last row pointer entry must match data length"));
  for (uint64_t k = 0; k < indices_len; ++k)
    if (indices[k] >= ncols) return set_err(err, E_VALUE, value_msg("Column index out of bounds"));
  return ok(err);
}

// CsrArray::check_sorted_indices, csr_array.rs:221-233
bool check_sorted_indices(const uint64_t* indices, uint64_t indices_len, const uint64_t* indptr,
                          uint64_t indptr_len) {
  for (uint64_t row = 0; row + 1 < indptr_len; ++row) {
    uint64_t start = indptr[row], end = indptr[row + 1];
    uint64_t stop = end > 0 ? end - 1 : 0;  // saturating_sub(1)
    for (uint64_t i = start; i < stop; ++i)
      if (i + 1 < indices_len && indices[i] > indices[i + 1]) return false;
  }
  return true;
}

// CsrArray::new validation, csr_array.rs:77-136
int csr_array_new_check(const uint64_t* indptr, uint64_t indptr_len, const uint64_t* indices,
                        uint64_t indices_len, uint64_t data_len, uint64_t nrows, uint64_t ncols,
                        int* sorted, or_err* err) {
  if (data_len != indices_len)
    return set_err(err, E_INCONSISTENT_DATA,
                   incons_msg("data and indices must have the same length"));
  if (indptr_len != nrows + 1)
    return set_err(err, E_INCONSISTENT_DATA,
                   incons_msg("indptr length (" + std::to_string(indptr_len) +
                              ") must be one more than the number of rows (" +
                              std::to_string(nrows) + ")"));
  if (indices_len > 0) {
    uint64_t mx = 0;
    for (uint64_t k = 0; k < indices_len; ++k) mx = std::max(mx, indices[k]);
    if (mx >= ncols)
      return set_err(err, E_INDEX_OUT_OF_BOUNDS,
                     "Index (0, " + std::to_string(mx) + ") out of bounds for array with shape (" +
                         std::to_string(nrows) + ", " + std::to_string(ncols) + ")",
                     0, mx, nrows, ncols);
  }
  if (indptr_len > 0) {
    uint64_t first = indptr[0], last = indptr[indptr_len - 1];
    if (first != 0)
      return set_err(err, E_INCONSISTENT_DATA, incons_msg("first element of indptr must be 0"));
    if (last != data_len)
      return set_err(err, E_INCONSISTENT_DATA,
                     incons_msg("last element of indptr (" + std::to_string(last) +
                                ") must equal data length (" + std::to_string(data_len) + ")"));
  }
  if (sorted) *sorted = check_sorted_indices(indices, indices_len, indptr, indptr_len) ? 1 : 0;
  return ok(err);
}

// CsrArray::from_triplets, csr_array.rs:152-219
template <class T>
int csr_array_from_triplets(const uint64_t* rows, const uint64_t* cols, const T* data,
                            uint64_t nnz, uint64_t nrows, uint64_t ncols, int sorted,
                            uint64_t* indptr, uint64_t* indices, T* out, int* has_sorted,
                            or_err* err) {
  if (nnz == 0) {
    for (uint64_t i = 0; i <= nrows; ++i) indptr[i] = 0;
    return csr_array_new_check(indptr, nrows + 1, indices, 0, 0, nrows, ncols, has_sorted, err);
  }
  for (uint64_t k = 0; k < nnz; ++k)
    if (rows[k] >= nrows || cols[k] >= ncols)
      return set_err(err, E_INDEX_OUT_OF_BOUNDS,
                     "Index (" + std::to_string(rows[k]) + ", " + std::to_string(cols[k]) +
                         ") out of bounds for array with shape (" + std::to_string(nrows) + ", " +
                         std::to_string(ncols) + ")",
                     rows[k], cols[k], nrows, ncols);
  std::vector<uint64_t> perm(nnz);
  std::iota(perm.begin(), perm.end(), 0);
  if (!sorted)
    std::stable_sort(perm.begin(), perm.end(), [&](uint64_t a, uint64_t b) {
      if (rows[a] != rows[b]) return rows[a] < rows[b];
      return cols[a] < cols[b];
    });
  std::vector<uint64_t> counts(nrows, 0);
  for (uint64_t k = 0; k < nnz; ++k) counts[rows[k]] += 1;
  indptr[0] = 0;
  uint64_t cum = 0;
  for (uint64_t i = 0; i < nrows; ++i) { cum += counts[i]; indptr[i + 1] = cum; }
  for (uint64_t k = 0; k < nnz; ++k) {
    indices[k] = cols[perm[k]];
    out[k] = data[perm[k]];
  }
  return csr_array_new_check(indptr, nrows + 1, indices, nnz, nnz, nrows, ncols, has_sorted, err);
}

// CsrMatrix::transpose (counting sort), csr.rs:289-326.  Column counts run
// over the whole indices array, exactly as the reference does, and slots no
// row range reaches keep (0, 0).  CsrArray::transpose (csr_array.rs:595-625)
// produces the same arrays through a stable sort of swapped triplets.
template <class T>
void csr_transpose(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t nrows,
                   uint64_t ncols, uint64_t* indptr_t, uint64_t* indices_t, T* data_t) {
  // The reference counts over indices.len(), which equals indptr[nrows] for
  // every matrix its constructors accept (from_raw_csr checks last == len).
  std::vector<uint64_t> counts(ncols, 0);
  for (uint64_t k = 0; k < indptr[nrows]; ++k) counts[indices[k]] += 1;
  indptr_t[0] = 0;
  for (uint64_t c = 0; c < ncols; ++c) indptr_t[c + 1] = indptr_t[c] + counts[c];
  uint64_t total = indptr_t[ncols];
  for (uint64_t k = 0; k < total; ++k) { indices_t[k] = 0; data_t[k] = T(0); }
  std::fill(counts.begin(), counts.end(), 0);
  for (uint64_t r = 0; r < nrows; ++r)
    for (uint64_t k = indptr[r]; k < indptr[r + 1]; ++k) {
      uint64_t c = indices[k];
      uint64_t dst = indptr_t[c] + counts[c];
      indices_t[dst] = r;
      data_t[dst] = data[k];
      counts[c] += 1;
    }
}

// CsrMatrix::get, csr.rs:33-48: first match in storage order
template <class T>
T csr_get(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t nrows,
          uint64_t ncols, uint64_t i, uint64_t j) {
  if (i >= nrows || j >= ncols) return T(0);
  for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k)
    if (indices[k] == j) return data[k];
  return T(0);
}

// CsrArray::dot_vector (csr_array.rs:569-593), CsrMatrix::dot (csr.rs:479-497)
// and MatrixLinearOperator::matvec (interface.rs:257-279) are the same loop:
// sum starts at zero, then sum = sum + a*x in storage order.  A row whose
// end precedes its start (possible through CsrArray::new) is empty.
template <class T, class IP, class IX>
void spmv(const IP* indptr, const IX* indices, const T* data, uint64_t nrows, const T* x, T* y) {
  par_for((int64_t)nrows, [=](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      T sum = T(0);
      for (IP k = indptr[i]; k < indptr[i + 1]; ++k) sum = sum + data[k] * x[indices[k]];
      y[i] = sum;
    }
  });
}

// iterative.rs:827-834: `.sum()` of f32/f64 folds from -0.0 in current Rust
template <class F>
F dot(const std::vector<F>& a, const std::vector<F>& b) {
  F s = F(-0.0);
  for (size_t i = 0; i < a.size(); ++i) s = s + a[i] * b[i];
  return s;
}
template <class F>
F norm2(const std::vector<F>& a) {
  return std::sqrt(dot(a, a));
}

}  // namespace

// ---------------------------------------------------------------- operators
struct or_op {
  virtual ~or_op() {}
  int f64 = 1;
  uint64_t nrows = 0, ncols = 0;
  virtual void mv64(const double* x, double* y) const = 0;
  virtual void mv32(const float* x, float* y) const = 0;
  // rmatvec: the preconditioners and elementwise operators are their own
  // adjoints (interface.rs:86-88, :121-124, :164-167; preconditioners.rs:88-91;
  // ic.rs:227-230)
  virtual void rmv64(const double* x, double* y) const { mv64(x, y); }
  virtual void rmv32(const float* x, float* y) const { mv32(x, y); }
};

namespace {

template <class F>
void op_matvec(const or_op* op, const F* x, F* y);
template <>
void op_matvec<double>(const or_op* op, const double* x, double* y) { op->mv64(x, y); }
template <>
void op_matvec<float>(const or_op* op, const float* x, float* y) { op->mv32(x, y); }

template <class F>
std::vector<F> op_apply(const or_op* op, const std::vector<F>& x) {
  std::vector<F> y(op->nrows);
  op_matvec<F>(op, x.data(), y.data());
  return y;
}
template <class F>
std::vector<F> op_rapply(const or_op* op, const std::vector<F>& x) {
  std::vector<F> y(op->ncols);
  if constexpr (sizeof(F) == 8) op->rmv64((const double*)x.data(), (double*)y.data());
  else op->rmv32((const float*)x.data(), (float*)y.data());
  return y;
}

// MatrixLinearOperator<F, CsrMatrix<F>> (interface.rs:232-296)
struct CsrOp : or_op {
  std::vector<uint64_t> indptr, indices;
  std::vector<double> d64;
  std::vector<float> d32;
  void mv64(const double* x, double* y) const override {
    spmv<double>(indptr.data(), indices.data(), d64.data(), nrows, x, y);
  }
  void mv32(const float* x, float* y) const override {
    spmv<float>(indptr.data(), indices.data(), d32.data(), nrows, x, y);
  }
  // MatrixLinearOperator::rmatvec (interface.rs:281-285): the transposed
  // matrix's matvec, transpose built once
  mutable std::vector<uint64_t> tptr, tidx;
  mutable std::vector<double> t64;
  mutable std::vector<float> t32;
  void build_t() const {
    if (!tptr.empty()) return;
    const uint64_t nnz = indptr[nrows];
    tptr.assign(ncols + 1, 0);
    tidx.resize(nnz);
    t64.resize(nnz);
    t32.resize(nnz);
    for (uint64_t k = 0; k < nnz; ++k) tptr[indices[k] + 1] += 1;
    for (uint64_t c = 0; c < ncols; ++c) tptr[c + 1] += tptr[c];
    std::vector<uint64_t> cur(tptr.begin(), tptr.end() - 1);
    for (uint64_t r = 0; r < nrows; ++r)
      for (uint64_t k = indptr[r]; k < indptr[r + 1]; ++k) {
        const uint64_t o = cur[indices[k]]++;
        tidx[o] = r;
        t64[o] = d64[k];
        t32[o] = d32[k];
      }
  }
  void rmv64(const double* x, double* y) const override {
    build_t();
    spmv<double>(tptr.data(), tidx.data(), t64.data(), ncols, x, y);
  }
  void rmv32(const float* x, float* y) const override {
    build_t();
    spmv<float>(tptr.data(), tidx.data(), t32.data(), ncols, x, y);
  }
};

// IdentityOperator (interface.rs:55-93)
struct IdentityOp : or_op {
  void mv64(const double* x, double* y) const override { std::memcpy(y, x, nrows * 8); }
  void mv32(const float* x, float* y) const override { std::memcpy(y, x, nrows * 4); }
};

// ScaledIdentityOperator (interface.rs:95-130): x_i * scale
struct ScaledIdentityOp : or_op {
  double s64 = 1; float s32 = 1;
  void mv64(const double* x, double* y) const override {
    for (uint64_t i = 0; i < nrows; ++i) y[i] = x[i] * s64;
  }
  void mv32(const float* x, float* y) const override {
    for (uint64_t i = 0; i < nrows; ++i) y[i] = x[i] * s32;
  }
};

// DiagonalOperator (interface.rs:132-175) and the apply of
// JacobiPreconditioner (preconditioners.rs:64-82): y_i = x_i * d_i
struct DiagOp : or_op {
  std::vector<double> d64;
  std::vector<float> d32;
  void mv64(const double* x, double* y) const override {
    const double* d = d64.data();
    par_for((int64_t)nrows, [=](int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i) y[i] = x[i] * d[i];
    });
  }
  void mv32(const float* x, float* y) const override {
    const float* d = d32.data();
    par_for((int64_t)nrows, [=](int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i) y[i] = x[i] * d[i];
    });
  }
};

// IC0Preconditioner (ic.rs:15-230)
template <class F>
struct IC0Data {
  std::vector<uint64_t> indptr, indices;
  std::vector<F> data;
  // transposed factor for the backward solve: for column i, the rows j > i
  // whose FIRST entry with column i is taken (ic.rs:199-214 breaks at it)
  std::vector<uint64_t> tptr, trow;
  std::vector<F> tval;
  std::vector<F> diag_first;  // first diagonal entry per row (ic.rs:185-191)
};

template <class F>
int ic0_factor(const CsrOp* a, IC0Data<F>& L, or_err* err) {
  const uint64_t n = a->nrows;
  if (n != a->ncols)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(n, a->ncols), n, a->ncols);
  const F* ad = nullptr;
  if constexpr (sizeof(F) == 8) ad = a->d64.data(); else ad = a->d32.data();
  // lower-triangular copy in storage order (ic.rs:32-49)
  L.indptr.assign(1, 0);
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t k = a->indptr[i]; k < a->indptr[i + 1]; ++k) {
      uint64_t j = a->indices[k];
      if (j <= i) { L.indices.push_back(j); L.data.push_back(ad[k]); }
    }
    L.indptr.push_back(L.indices.size());
  }
  auto& li = L.indices;
  auto& ld = L.data;
  auto& lp = L.indptr;
  // factorisation loop (ic.rs:52-129)
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t rs = lp[i], re = lp[i + 1];
    uint64_t di = UINT64_MAX;
    for (uint64_t k = rs; k < re; ++k)
      if (li[k] == i) { di = k; break; }
    if (di == UINT64_MAX)
      return set_err(err, E_VALUE,
                     value_msg("Missing diagonal element at position " + std::to_string(i)));
    F dv = ld[di];
    for (uint64_t k = rs; k < di; ++k) {
      uint64_t j = li[k];
      F ljj = F(0);
      for (uint64_t q = lp[j]; q < lp[j + 1]; ++q)
        if (li[q] == j) { ljj = ld[q]; break; }
      dv -= ld[k] * ld[k] / ljj;
    }
    if (dv <= F(0))
      return set_err(err, E_VALUE,
                     value_msg("Matrix is not positive definite or factorization broke down"));
    ld[di] = std::sqrt(dv);
    for (uint64_t k = di + 1; k < re; ++k) {
      uint64_t j = li[k];
      F sum = F(0);
      for (uint64_t p = rs; p < di; ++p) {
        uint64_t cp = li[p];
        for (uint64_t q = lp[j]; q < lp[j + 1]; ++q)
          if (li[q] == cp) { sum += ld[p] * ld[q]; break; }
      }
      ld[k] = (ld[k] - sum) / ld[di];
    }
  }
  // CsrMatrix::from_raw_csr on the factor (ic.rs:132) cannot fail here:
  // indptr is monotone by construction and every column is <= its row.
  // Backward-solve helpers.
  L.diag_first.assign(n, F(1));
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t k = lp[i]; k < lp[i + 1]; ++k)
      if (li[k] == i) { L.diag_first[i] = ld[k]; break; }
  std::vector<uint64_t> cnt(n + 1, 0);
  std::vector<char> seen;
  // first occurrence of (row j, column c) for c < j
  std::vector<uint64_t> first_k;
  for (uint64_t j = 0; j < n; ++j) {
    for (uint64_t k = lp[j]; k < lp[j + 1]; ++k) {
      uint64_t c = li[k];
      if (c >= j) continue;
      bool dup = false;
      for (uint64_t q = lp[j]; q < k; ++q)
        if (li[q] == c) { dup = true; break; }
      if (!dup) { cnt[c + 1] += 1; first_k.push_back(k); }
    }
  }
  for (uint64_t c = 0; c < n; ++c) cnt[c + 1] += cnt[c];
  L.tptr = cnt;
  L.trow.assign(cnt[n], 0);
  L.tval.assign(cnt[n], F(0));
  std::vector<uint64_t> fill(n, 0);
  // first_k is in ascending row order, so each column list is ascending in j
  uint64_t fk = 0;
  for (uint64_t j = 0; j < n; ++j) {
    for (uint64_t k = lp[j]; k < lp[j + 1]; ++k) {
      if (fk < first_k.size() && first_k[fk] == k) {
        uint64_t c = li[k];
        uint64_t dst = L.tptr[c] + fill[c]++;
        L.trow[dst] = j;
        L.tval[dst] = ld[k];
        ++fk;
      }
    }
  }
  return ok(err);
}

template <class F>
void ic0_apply(const IC0Data<F>& L, uint64_t n, const F* x, F* y, bool fast) {
  // forward solve L z = x (ic.rs:154-174): the LAST diagonal entry wins
  std::vector<F> z(n, F(0));
  for (uint64_t i = 0; i < n; ++i) {
    F sum = x[i];
    F dv = F(1);
    for (uint64_t k = L.indptr[i]; k < L.indptr[i + 1]; ++k) {
      uint64_t j = L.indices[k];
      F v = L.data[k];
      if (j < i) sum -= v * z[j];
      else if (j == i) dv = v;
    }
    z[i] = sum / dv;
  }
  // backward solve L^T y = z (ic.rs:177-217): first diagonal entry; for each
  // j > i in ascending order, the first entry of row j in column i
  for (uint64_t ii = n; ii-- > 0;) {
    F sum = z[ii];
    if (fast) {
      for (uint64_t t = L.tptr[ii]; t < L.tptr[ii + 1]; ++t) sum -= L.tval[t] * y[L.trow[t]];
    } else {
      for (uint64_t j = ii + 1; j < n; ++j)
        for (uint64_t k = L.indptr[j]; k < L.indptr[j + 1]; ++k)
          if (L.indices[k] == ii) { sum -= L.data[k] * y[j]; break; }
    }
    y[ii] = sum / L.diag_first[ii];
  }
}

struct IC0Op : or_op {
  IC0Data<double> l64;
  IC0Data<float> l32;
  bool fast = true;
  void mv64(const double* x, double* y) const override { ic0_apply(l64, nrows, x, y, fast); }
  void mv32(const float* x, float* y) const override { ic0_apply(l32, nrows, x, y, fast); }
};

// ILU0Preconditioner (preconditioners.rs:194-399): factorisation with k
// outermost as the reference writes it, then the L / U split and the two
// substitutions.
template <class F>
struct ILU0Data {
  std::vector<uint64_t> lp, li, up, ui;
  std::vector<F> ld, ud;
};
template <class F>
int ilu0_factor(const CsrOp* a, ILU0Data<F>& out, or_err* err) {
  const uint64_t n = a->nrows;
  const auto& indptr = a->indptr;
  const auto& indices = a->indices;
  std::vector<F> data(indices.size());
  for (size_t q = 0; q < data.size(); ++q) data[q] = sizeof(F) == 8 ? (F)a->d64[q] : (F)a->d32[q];
  const F eps = std::numeric_limits<F>::epsilon();
  for (uint64_t k = 0; k < n; ++k) {
    // find_diagonal_index (preconditioners.rs:382-399)
    int64_t kd = -1;
    for (uint64_t q = indptr[k]; q < indptr[k + 1]; ++q)
      if (indices[q] == k) { kd = (int64_t)q; break; }
    if (kd < 0) return set_err(err, E_VALUE, value_msg("Missing diagonal element at row " + std::to_string(k)));
    const F kdiag = data[kd];
    if (std::fabs(kdiag) < eps) return set_err(err, E_VALUE, value_msg("Zero pivot at position " + std::to_string(k)));
    for (uint64_t i = k + 1; i < n; ++i) {
      const uint64_t rs = indptr[i], re = indptr[i + 1];
      int64_t kpos = -1;
      for (uint64_t q = rs; q < re; ++q) {
        if (indices[q] == k) { kpos = (int64_t)q; break; }
        if (indices[q] > k) break;
      }
      if (kpos < 0) continue;
      const F mult = data[kpos] / kdiag;
      data[kpos] = mult;
      for (uint64_t kj = indptr[k]; kj < indptr[k + 1]; ++kj) {
        const uint64_t j = indices[kj];
        if (j <= k) continue;
        for (uint64_t ij = rs; ij < re; ++ij)
          if (indices[ij] == j) { data[ij] = data[ij] - mult * data[kj]; break; }
      }
    }
  }
  out.lp.assign(1, 0);
  out.up.assign(1, 0);
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t q = indptr[i]; q < indptr[i + 1]; ++q) {
      if (indices[q] < i) { out.li.push_back(indices[q]); out.ld.push_back(data[q]); }
      else { out.ui.push_back(indices[q]); out.ud.push_back(data[q]); }
    }
    out.lp.push_back(out.li.size());
    out.up.push_back(out.ui.size());
  }
  return ok(err);
}
template <class F>
void ilu0_apply(const ILU0Data<F>& f, uint64_t n, const F* x, F* z) {
  std::vector<F> y(n);
  for (uint64_t i = 0; i < n; ++i) {
    y[i] = x[i];
    for (uint64_t q = f.lp[i]; q < f.lp[i + 1]; ++q) y[i] = y[i] - f.ld[q] * y[f.li[q]];
  }
  for (uint64_t t = n; t-- > 0;) {
    z[t] = y[t];
    F dv = F(1);
    for (uint64_t q = f.up[t]; q < f.up[t + 1]; ++q) {
      const uint64_t c = f.ui[q];
      if (c == t) dv = f.ud[q];
      else if (c > t) z[t] = z[t] - f.ud[q] * z[c];
    }
    z[t] /= dv;
  }
}
struct ILU0Op : or_op {
  ILU0Data<double> f64d;
  ILU0Data<float> f32d;
  void mv64(const double* x, double* y) const override { ilu0_apply(f64d, nrows, x, y); }
  void mv32(const float* x, float* y) const override { ilu0_apply(f32d, nrows, x, y); }
};

// SSORPreconditioner (preconditioners.rs:94-192)
template <class F>
void ssor_apply(const CsrOp* a, const std::vector<F>& dg, F omega, const F* x, F* w) {
  const uint64_t n = a->nrows;
  auto val = [&](uint64_t q) -> F { return sizeof(F) == 8 ? (F)a->d64[q] : (F)a->d32[q]; };
  std::vector<F> y(n), z(n);
  for (uint64_t i = 0; i < n; ++i) {
    F sum = x[i];
    for (uint64_t q = a->indptr[i]; q < a->indptr[i + 1]; ++q)
      if (a->indices[q] < i) sum -= omega * val(q) * y[a->indices[q]];
    y[i] = sum / dg[i];
  }
  for (uint64_t i = 0; i < n; ++i) z[i] = y[i] * dg[i];
  for (uint64_t t = n; t-- > 0;) {
    F sum = z[t];
    for (uint64_t q = a->indptr[t]; q < a->indptr[t + 1]; ++q)
      if (a->indices[q] > t) sum -= omega * val(q) * w[a->indices[q]];
    w[t] = sum / dg[t];
  }
}
struct SSOROp : or_op {
  const CsrOp* a = nullptr;
  std::vector<double> d64;
  std::vector<float> d32;
  double om64 = 1;
  float om32 = 1;
  void mv64(const double* x, double* y) const override { ssor_apply<double>(a, d64, om64, x, y); }
  void mv32(const float* x, float* y) const override { ssor_apply<float>(a, d32, om32, x, y); }
};

// M^-1 = G G^T: y = G (G^T x), G^T kept explicitly through the counting-sort
// transpose; both products are plain CSR SpMVs.
struct FsaiOp : or_op {
  std::vector<uint64_t> gp, gi, tp, ti;
  std::vector<double> g64, t64;
  std::vector<float> g32, t32;
  void mv64(const double* x, double* y) const override {
    std::vector<double> w(nrows);
    spmv<double>(tp.data(), ti.data(), t64.data(), nrows, x, w.data());
    spmv<double>(gp.data(), gi.data(), g64.data(), nrows, w.data(), y);
  }
  void mv32(const float* x, float* y) const override {
    std::vector<float> w(nrows);
    spmv<float>(tp.data(), ti.data(), t32.data(), nrows, x, w.data());
    spmv<float>(gp.data(), gi.data(), g32.data(), nrows, w.data(), y);
  }
};

// ------------------------------------------------------------------ solvers
template <class F>
struct SolveOut {
  std::vector<F> x;
  uint64_t iterations = 0;
  F residual_norm = F(0);
  bool converged = false;
  int message = M_MAX_ITER;
  int stalled = 0;  // gmres: a cycle that cannot advance (the reference loops forever)
};

template <class F>
F eps10() { return std::numeric_limits<F>::epsilon() * F(10); }

// cg, iterative.rs:40-162
template <class F>
SolveOut<F> cg(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
               const F* x0, const or_op* m) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r(n);
  for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  std::vector<F> z = m ? op_apply(m, r) : r;
  std::vector<F> p = z;
  F rz_old = dot(r, z);
  F bnorm = norm2(b);
  F tol = std::fmax(atol, rtol * bnorm);
  uint64_t it = 0;
  while (it < max_iter) {
    std::vector<F> ap = op_apply(a, p);
    F pap = dot(p, ap);
    if (pap <= F(0)) {
      o.x = x; o.iterations = it; o.residual_norm = norm2(r); o.converged = false;
      o.message = M_NOT_PD;
      return o;
    }
    F alpha = rz_old / pap;
    {
      F *xp = x.data(), *rp = r.data();
      const F *pp = p.data(), *app = ap.data();
      par_for((int64_t)n, [=](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) xp[i] += alpha * pp[i];
        for (int64_t i = lo; i < hi; ++i) rp[i] -= alpha * app[i];
      });
    }
    F rnorm = norm2(r);
    if (rnorm <= tol) {
      o.x = x; o.iterations = it + 1; o.residual_norm = rnorm; o.converged = true;
      o.message = M_CONVERGED;
      return o;
    }
    z = m ? op_apply(m, r) : r;
    F rz_new = dot(r, z);
    F beta = rz_new / rz_old;
    {
      F* pp = p.data();
      const F* zp = z.data();
      par_for((int64_t)n, [=](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) pp[i] = zp[i] + beta * pp[i];
      });
    }
    rz_old = rz_new;
    ++it;
  }
  o.x = x; o.iterations = it; o.residual_norm = norm2(r); o.converged = false;
  o.message = M_MAX_ITER;
  return o;
}

// bicgstab, iterative.rs:377-611 (left preconditioner M1 applied to p and
// s; right preconditioner M2 applied to v, t and to x every iteration)
template <class F>
SolveOut<F> bicgstab(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
                     const F* x0, const or_op* m1, const or_op* m2) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r(n);
  for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  F rnorm = norm2(r);
  F bnorm = norm2(b);
  F tol = std::fmax(atol, rtol * bnorm);
  auto finish = [&](uint64_t it, F res, bool conv, int msg) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv; o.message = msg;
    return o;
  };
  if (rnorm <= tol) return finish(0, rnorm, true, M_CONVERGED_INITIAL);
  std::vector<F> r_hat = r;
  std::vector<F> v(n, F(0)), p(n, F(0)), y(n, F(0)), s(n, F(0)), t;
  F rho_old = F(1), alpha = F(0), omega = F(1);
  uint64_t it = 0;
  const F e10 = eps10<F>();
  while (it < max_iter) {
    F rho = dot(r_hat, r);
    if (std::fabs(rho) < e10) return finish(it, rnorm, false, M_BD_RHO);
    F beta = (rho / rho_old) * (alpha / omega);
    for (uint64_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
    std::vector<F> p_t = m1 ? op_apply(m1, p) : p;
    v = op_apply(a, p_t);
    if (m2) v = op_apply(m2, v);
    F den = dot(r_hat, v);
    if (std::fabs(den) < e10) return finish(it, rnorm, false, M_BD_RHAT_V);
    alpha = rho / den;
    if (!std::isfinite(alpha)) return finish(it, rnorm, false, M_BD_ALPHA);
    for (uint64_t i = 0; i < n; ++i) {
      y[i] = x[i] + alpha * p_t[i];
      s[i] = r[i] - alpha * v[i];
    }
    F snorm = norm2(s);
    if (snorm <= tol) {
      x = y;
      if (m2) x = op_apply(m2, x);
      return finish(it + 1, snorm, true, M_CONVERGED);
    }
    std::vector<F> s_t = m1 ? op_apply(m1, s) : s;
    t = op_apply(a, s_t);
    if (m2) t = op_apply(m2, t);
    F ts = dot(t, s);
    F tt = dot(t, t);
    if (tt < e10) return finish(it, rnorm, false, M_BD_TT);
    omega = ts / tt;
    if (!std::isfinite(omega) || std::fabs(omega) < e10)
      return finish(it, rnorm, false, M_BD_OMEGA);
    for (uint64_t i = 0; i < n; ++i) {
      x[i] = y[i] + omega * s_t[i];
      r[i] = s[i] - omega * t[i];
    }
    if (m2) x = op_apply(m2, x);
    rnorm = norm2(r);
    if (rnorm <= tol) return finish(it + 1, rnorm, true, M_CONVERGED);
    rho_old = rho;
    ++it;
  }
  return finish(it, rnorm, false, M_MAX_ITER);
}

// gmres, iterative.rs:641-816: left-preconditioned restarted GMRES with
// modified Gram-Schmidt and Givens rotations.  On a happy breakdown the
// column being built is dropped (the loop breaks before the rotation and
// before inner_iter is advanced).  A cycle that ends with inner_iter = 0
// (restart = 0, or a breakdown at the first step: A r0 parallel to r0, as
// for A = c I) leaves x, r and the iteration count as they were, so the
// reference's loop repeats it forever; here the solve stops (stalled).
template <class F>
SolveOut<F> gmres(const or_op* a, const std::vector<F>& b, uint64_t max_iter, uint64_t restart_opt,
                  F rtol, F atol, const F* x0, const or_op* m) {
  const uint64_t n = a->nrows;
  const uint64_t restart = std::min(restart_opt, n);
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r(n);
  for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  if (m) r = op_apply(m, r);
  F rnorm = norm2(r);
  F bnorm = norm2(b);
  F tol = std::fmax(atol, rtol * bnorm);
  uint64_t outer = 0;
  const F e10 = eps10<F>();
  while (outer < max_iter && rnorm > tol) {
    std::vector<std::vector<F>> v(restart + 1, std::vector<F>(n, F(0)));
    std::vector<std::vector<F>> h(restart + 1, std::vector<F>(restart, F(0)));
    std::vector<F> cs(restart, F(0)), sn(restart, F(0)), s(restart + 1, F(0));
    for (uint64_t i = 0; i < n; ++i) v[0][i] = r[i] / rnorm;
    s[0] = rnorm;
    uint64_t j = 0;
    while (j < restart && j + outer < max_iter) {
      std::vector<F> w = op_apply(a, v[j]);
      if (m) w = op_apply(m, w);
      for (uint64_t i = 0; i <= j; ++i) {
        h[i][j] = dot(v[i], w);
        for (uint64_t k = 0; k < n; ++k) w[k] -= h[i][j] * v[i][k];
      }
      h[j + 1][j] = norm2(w);
      if (h[j + 1][j] < e10) break;
      for (uint64_t k = 0; k < n; ++k) v[j + 1][k] = w[k] / h[j + 1][j];
      for (uint64_t i = 0; i < j; ++i) {
        F temp = cs[i] * h[i][j] + sn[i] * h[i + 1][j];
        h[i + 1][j] = -sn[i] * h[i][j] + cs[i] * h[i + 1][j];
        h[i][j] = temp;
      }
      F rho = std::sqrt(h[j][j] * h[j][j] + h[j + 1][j] * h[j + 1][j]);
      cs[j] = h[j][j] / rho;
      sn[j] = h[j + 1][j] / rho;
      h[j][j] = rho;
      h[j + 1][j] = F(0);
      F temp = cs[j] * s[j] + sn[j] * s[j + 1];
      s[j + 1] = -sn[j] * s[j] + cs[j] * s[j + 1];
      s[j] = temp;
      ++j;
      if (std::fabs(s[j]) <= tol) break;
    }
    std::vector<F> yv(j, F(0));
    for (uint64_t ii = j; ii-- > 0;) {
      yv[ii] = s[ii];
      for (uint64_t q = ii + 1; q < j; ++q) yv[ii] = yv[ii] - h[ii][q] * yv[q];
      yv[ii] /= h[ii][ii];
    }
    for (uint64_t ii = 0; ii < j; ++ii)
      for (uint64_t k = 0; k < n; ++k) x[k] += yv[ii] * v[ii][k];
    ax = op_apply(a, x);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
    if (m) r = op_apply(m, r);
    rnorm = norm2(r);
    outer += j;
    if (rnorm <= tol) break;
    if (j == 0) {
      o.stalled = 1;
      break;
    }
  }
  o.x = x;
  o.iterations = outer;
  o.residual_norm = rnorm;
  o.converged = rnorm <= tol;
  o.message = o.converged ? M_CONVERGED : M_MAX_ITER;
  return o;
}


// bicg, iterative.rs:189-345: left preconditioner on r (and on A^T p*),
// right preconditioner on r* (and on A p); no initial convergence test
template <class F>
SolveOut<F> bicg(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
                 const F* x0, const or_op* m1, const or_op* m2) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r(n);
  for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  std::vector<F> rs = r;
  std::vector<F> z = m1 ? op_apply(m1, r) : r;
  std::vector<F> zs = m2 ? op_apply(m2, rs) : rs;
  std::vector<F> p = z, ps = zs;
  F rho_old = dot(rs, z);
  F bnorm = norm2(b);
  F tol = std::fmax(atol, rtol * bnorm);
  auto finish = [&](uint64_t it, F res, bool conv, int msg) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv; o.message = msg;
    return o;
  };
  const F e10 = eps10<F>();
  uint64_t it = 0;
  while (it < max_iter) {
    std::vector<F> q = op_apply(a, p);
    if (m2) q = op_apply(m2, q);
    std::vector<F> qs = op_rapply(a, ps);
    if (m1) qs = op_apply(m1, qs);
    F den = dot(ps, q);
    if (std::fabs(den) < e10) return finish(it, norm2(r), false, M_BICG_PQ);
    F alpha = rho_old / den;
    for (uint64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      rs[i] -= alpha * qs[i];
    }
    F rnorm = norm2(r);
    if (rnorm <= tol) return finish(it + 1, rnorm, true, M_CONVERGED);
    z = m1 ? op_apply(m1, r) : r;
    zs = m2 ? op_apply(m2, rs) : rs;
    F rho = dot(rs, z);
    if (std::fabs(rho) < e10) return finish(it + 1, rnorm, false, M_BICG_RHO);
    F beta = rho / rho_old;
    for (uint64_t i = 0; i < n; ++i) {
      p[i] = z[i] + beta * p[i];
      ps[i] = zs[i] + beta * ps[i];
    }
    rho_old = rho;
    ++it;
  }
  return finish(it, norm2(r), false, M_MAX_ITER);
}

// cgs, cgs.rs:15-193: right preconditioner applied to p, u + q and q
template <class F>
SolveOut<F> cgs(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
                const F* x0, const or_op* m) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r(n);
  for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  F rnorm = norm2(r);
  F bnorm = norm2(b);
  F tol = std::fmax(atol, rtol * bnorm);
  auto finish = [&](uint64_t it, F res, bool conv, int msg) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv; o.message = msg;
    return o;
  };
  if (rnorm <= tol) return finish(0, rnorm, true, M_CONVERGED_INITIAL);
  std::vector<F> rt = r, u(n, F(0)), p(n, F(0)), q(n, F(0)), uq(n);
  F rho = F(1);
  const F e10 = eps10<F>();
  uint64_t it = 0;
  while (it < max_iter) {
    F rho_new = dot(rt, r);
    if (std::fabs(rho_new) < e10) return finish(it, rnorm, false, M_CGS_RHO);
    F beta = it == 0 ? F(0) : rho_new / rho;
    for (uint64_t i = 0; i < n; ++i) {
      u[i] = r[i] + beta * q[i];
      p[i] = u[i] + beta * (q[i] + beta * p[i]);
    }
    std::vector<F> pp = m ? op_apply(m, p) : p;
    std::vector<F> v = op_apply(a, pp);
    F sigma = dot(rt, v);
    if (std::fabs(sigma) < e10) return finish(it, rnorm, false, M_CGS_SIGMA);
    F alpha = rho_new / sigma;
    for (uint64_t i = 0; i < n; ++i) q[i] = u[i] - alpha * v[i];
    for (uint64_t i = 0; i < n; ++i) uq[i] = u[i] + q[i];
    std::vector<F> uqp = m ? op_apply(m, uq) : uq;
    for (uint64_t i = 0; i < n; ++i) x[i] += alpha * uqp[i];
    std::vector<F> qp = m ? op_apply(m, q) : q;
    std::vector<F> aq = op_apply(a, qp);
    for (uint64_t i = 0; i < n; ++i) r[i] -= alpha * (v[i] + aq[i]);
    rho = rho_new;
    ++it;
    rnorm = norm2(r);
    if (rnorm <= tol) break;
  }
  const bool conv = rnorm <= tol;
  return finish(it, rnorm, conv, conv ? M_CONVERGED : M_MAX_ITER);
}

// qmr, qmr.rs:44-259 (a BiCGSTAB-like recurrence with the transposed
// operator in the shadow sequence); tol = atol + rtol ||b||, strict tests
template <class F>
SolveOut<F> qmr(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
                const F* x0, const or_op* m1, const or_op* m2) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  bool all_zero = true;
  for (uint64_t i = 0; i < n; ++i) all_zero = all_zero && x[i] == F(0);
  std::vector<F> r(n);
  if (!all_zero) {
    std::vector<F> ax = op_apply(a, x);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
  } else {
    r = b;
  }
  if (m1) r = op_apply(m1, r);
  std::vector<F> rt = r;
  std::vector<F> p(n, F(0)), pt(n, F(0)), q(n, F(0)), qt(n, F(0)), s(n), t;
  F rho = F(1), rho_old, alpha = F(0), omega = F(1);
  F bnorm = norm2(b);
  F rnorm = norm2(r);
  F tol = atol + rtol * bnorm;
  auto finish = [&](uint64_t it, F res, bool conv, int msg) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv; o.message = msg;
    return o;
  };
  if (rnorm < tol) return finish(0, rnorm, true, M_QMR_INITIAL);
  const F e10 = eps10<F>();
  for (uint64_t it = 0; it < max_iter; ++it) {
    rho_old = rho;
    rho = dot(rt, r);
    if (std::fabs(rho) < e10) return finish(it, rnorm, false, M_QMR_RHO);
    F beta = it == 0 ? F(0) : (rho / rho_old) * (alpha / omega);
    if (it == 0) p = r;
    else for (uint64_t i = 0; i < n; ++i) p[i] = r[i] + (p[i] - q[i] * omega) * beta;
    std::vector<F> pp = m2 ? op_apply(m2, p) : p;
    q = op_apply(a, pp);
    if (m1) q = op_apply(m1, q);
    if (it == 0) pt = rt;
    else for (uint64_t i = 0; i < n; ++i) pt[i] = rt[i] + (pt[i] - qt[i] * omega) * beta;
    std::vector<F> ptp = m1 ? op_rapply(m1, pt) : pt;
    qt = op_rapply(a, ptp);
    if (m2) qt = op_rapply(m2, qt);
    F dpq = dot(pt, q);
    if (std::fabs(dpq) < e10) return finish(it, rnorm, false, M_QMR_PQ);
    alpha = rho / dpq;
    for (uint64_t i = 0; i < n; ++i) s[i] = r[i] - q[i] * alpha;
    std::vector<F> sp = m2 ? op_apply(m2, s) : s;
    t = op_apply(a, sp);
    if (m1) t = op_apply(m1, t);
    F tt = dot(t, t);
    omega = tt == F(0) ? F(0) : dot(t, s) / tt;
    for (uint64_t i = 0; i < n; ++i) x[i] = x[i] + pp[i] * alpha;
    for (uint64_t i = 0; i < n; ++i) x[i] = x[i] + sp[i] * omega;
    for (uint64_t i = 0; i < n; ++i) r[i] = s[i] - t[i] * omega;
    rnorm = norm2(r);
    if (rnorm < tol) return finish(it + 1, rnorm, true, M_QMR_CONVERGED);
    if (std::fabs(omega) < std::numeric_limits<F>::epsilon())
      return finish(it + 1, rnorm, false, M_QMR_OMEGA);
  }
  return finish(max_iter, rnorm, false, M_QMR_MAX_ITER);
}

// minres, minres.rs:66-257 (Paige-Saunders); error 1: "Indefinite
// preconditioner", error 2: "Non-symmetric matrix" (ComputationError)
template <class F>
SolveOut<F> minres(const or_op* a, const std::vector<F>& b, uint64_t max_iter, F rtol, F atol,
                   const F* x0, const or_op* m, int* error) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  *error = 0;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  auto finish = [&](uint64_t it, F res, bool conv, int msg) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv; o.message = msg;
    return o;
  };
  const F bnorm = norm2(b);
  if (bnorm < atol) return finish(0, F(0), true, M_ZERO_RHS);
  std::vector<F> ax = op_apply(a, x);
  std::vector<F> r1(n);
  for (uint64_t i = 0; i < n; ++i) r1[i] = b[i] - ax[i];
  std::vector<F> y = m ? op_apply(m, r1) : r1;
  F beta1_sq = dot(r1, y);
  if (beta1_sq < F(0)) { *error = 1; return o; }
  if (beta1_sq == F(0)) return finish(0, F(0), true, M_ZERO_RESIDUAL);
  F beta1 = std::sqrt(beta1_sq);
  F oldb = F(0), beta = beta1, dbar = F(0), epsln = F(0), phibar = beta1;
  F cs = F(-1), sn = F(0);
  std::vector<F> w(n, F(0)), w2(n, F(0)), r2 = r1, v(n, F(0)), w1;
  std::fill(r1.begin(), r1.end(), F(0));
  F tnorm2 = F(0), qrnorm = beta1;
  const F eps = std::numeric_limits<F>::epsilon();
  for (uint64_t itn = 0; itn < max_iter; ++itn) {
    const F s = F(1) / beta;
    for (uint64_t i = 0; i < n; ++i) v[i] = s * y[i];
    std::vector<F> yn = op_apply(a, v);
    if (itn >= 1)
      for (uint64_t i = 0; i < n; ++i) yn[i] -= (beta / oldb) * r1[i];
    F alfa = dot(v, yn);
    for (uint64_t i = 0; i < n; ++i) yn[i] -= (alfa / beta) * r2[i];
    r1 = r2;
    r2 = yn;
    y = m ? op_apply(m, r2) : r2;
    oldb = beta;
    F beta_sq = dot(r2, y);
    if (beta_sq < F(0)) { *error = 2; return o; }
    beta = std::sqrt(beta_sq);
    tnorm2 = tnorm2 + alfa * alfa + oldb * oldb + beta * beta;
    F oldeps = epsln;
    F delta = cs * dbar + sn * alfa;
    F gbar = sn * dbar - cs * alfa;
    epsln = sn * beta;
    dbar = -cs * beta;
    F gamma = std::sqrt(gbar * gbar + beta * beta);
    F gc = gamma > eps ? gamma : eps;
    cs = gbar / gc;
    sn = beta / gc;
    F phi = cs * phibar;
    phibar = sn * phibar;
    F denom = F(1) / gc;
    w1 = w2;
    w2 = w;
    for (uint64_t i = 0; i < n; ++i) {
      w[i] = (v[i] - oldeps * w1[i] - delta * w2[i]) * denom;
      x[i] += phi * w[i];
    }
    qrnorm = phibar;
    F rnorm = qrnorm;
    F anorm = std::sqrt(tnorm2);
    F ynorm = norm2(x);
    F test1 = (ynorm == F(0) || anorm == F(0)) ? std::numeric_limits<F>::infinity() : rnorm / (anorm * ynorm);
    if (test1 <= rtol || rnorm <= atol) return finish(itn + 1, rnorm, true, M_CONVERGED);
  }
  return finish(max_iter, qrnorm, false, M_MAX_ITER);
}

// lgmres, lgmres.rs:58-327: restarted left-preconditioned GMRES with
// classical Gram-Schmidt (each h_ij from the unorthogonalised w); the
// augmentation vectors are collected but unused, as in the reference
template <class F>
SolveOut<F> lgmres(const or_op* a, const std::vector<F>& b, uint64_t max_iter, uint64_t inner_m,
                   F rtol, F atol, const F* x0, const or_op* m) {
  const uint64_t n = a->nrows;
  SolveOut<F> o;
  std::vector<F> x(n, F(0));
  if (x0) x.assign(x0, x0 + n);
  auto finish = [&](uint64_t it, F res, bool conv) {
    o.x = x; o.iterations = it; o.residual_norm = res; o.converged = conv;
    o.message = conv ? M_CONVERGED : M_MAX_ITER;
    return o;
  };
  F bnorm = F(0);
  for (uint64_t i = 0; i < n; ++i) bnorm = bnorm + b[i] * b[i];
  bnorm = std::sqrt(bnorm);
  if (bnorm < atol) return finish(0, F(0), true);
  auto residual = [&]() {
    std::vector<F> ax = op_apply(a, x);
    std::vector<F> r(n);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
    return m ? op_apply(m, r) : r;
  };
  std::vector<F> r = residual();
  F rn = norm2(r);
  if (rn < atol || rn / bnorm < rtol) return finish(0, rn, true);
  const F eps = std::numeric_limits<F>::epsilon();
  uint64_t total = 0;
  for (uint64_t outer = 0; outer < max_iter; ++outer) {
    // inner_gmres (lgmres.rs:191-327)
    std::vector<F> xi(n, F(0));
    F r0n = norm2(r);
    if (!(r0n < eps)) {
      const uint64_t mm = inner_m;
      std::vector<std::vector<F>> v(mm + 1, std::vector<F>(n, F(0)));
      for (uint64_t i = 0; i < n; ++i) v[0][i] = r[i] / r0n;
      std::vector<std::vector<F>> h(mm + 1, std::vector<F>(mm, F(0)));
      std::vector<F> sv(mm + 1, F(0)), cv(mm + 1, F(0)), beta(mm + 2, F(0));
      beta[0] = r0n;
      uint64_t k = 0;
      for (uint64_t j = 0; j < mm; ++j) {
        std::vector<F> w = op_apply(a, v[j]);
        if (m) w = op_apply(m, w);
        std::vector<F> wo = w;
        for (uint64_t i = 0; i <= j; ++i) {
          F hij = dot(w, v[i]);
          h[i][j] = hij;
          for (uint64_t q = 0; q < n; ++q) wo[q] -= hij * v[i][q];
        }
        F hn = norm2(wo);
        if (hn > eps) {
          h[j + 1][j] = hn;
          for (uint64_t q = 0; q < n; ++q) v[j + 1][q] = wo[q] / hn;
        } else {
          k = j + 1;
          break;
        }
        for (uint64_t i = 0; i < j; ++i) {
          F temp = cv[i] * h[i][j] + sv[i] * h[i + 1][j];
          h[i + 1][j] = -sv[i] * h[i][j] + cv[i] * h[i + 1][j];
          h[i][j] = temp;
        }
        F hjj = h[j][j], hj1 = h[j + 1][j];
        F rho = std::sqrt(hjj * hjj + hj1 * hj1);
        if (rho > eps) {
          cv[j] = hjj / rho;
          sv[j] = hj1 / rho;
          h[j][j] = cv[j] * hjj + sv[j] * hj1;
          h[j + 1][j] = F(0);
          beta[j + 1] = -sv[j] * beta[j];
          beta[j] = cv[j] * beta[j];
          k = j + 1;
          if (std::fabs(beta[j + 1]) < F(1e-10)) break;
        } else {
          k = j;
          break;
        }
      }
      if (k > 0) {
        std::vector<F> y(k, F(0));
        for (uint64_t i = k; i-- > 0;) {
          y[i] = beta[i];
          for (uint64_t j = i + 1; j < k; ++j) y[i] = y[i] - h[i][j] * y[j];
          if (std::fabs(h[i][i]) > eps) y[i] /= h[i][i];
          else y[i] = F(0);
        }
        for (uint64_t i = 0; i < k; ++i)
          for (uint64_t q = 0; q < n; ++q) xi[q] += y[i] * v[i][q];
      }
    }
    for (uint64_t q = 0; q < n; ++q) x[q] += xi[q];
    ++total;
    r = residual();
    rn = norm2(r);
    if (rn < atol || rn / bnorm < rtol) return finish(total, rn, true);
  }
  return finish(total, rn, false);
}

template <class F>
void fill_result(const SolveOut<F>& s, void* x_out, or_result* res) {
  std::memcpy(x_out, s.x.data(), s.x.size() * sizeof(F));
  if (res) {
    res->iterations = s.iterations;
    res->residual_norm = (double)s.residual_norm;
    res->converged = s.converged ? 1 : 0;
    res->message = s.message;
  }
}

template <class F>
int check_square_and_len(const or_op* a, const char* solver, or_err* err) {
  if (a->nrows != a->ncols)
    return set_err(err, E_VALUE,
                   value_msg(std::string("Matrix must be square for ") + solver + " solver"));
  return 0;
}

}  // namespace

extern "C" {

// Host threads for the row-parallel SpMV and elementwise loops (>= 1).
void or_set_threads(int n) { pool().resize(n); }
int or_get_threads(void) { return pool().size(); }

int or_csr_matrix_new_f64(const double* data, const uint64_t* rows, const uint64_t* cols,
                          uint64_t nnz, uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                          uint64_t* indices_out, double* data_out, or_err* err) {
  return csr_matrix_new<double>(data, rows, cols, nnz, nrows, ncols, indptr_out, indices_out,
                                data_out, err);
}
int or_csr_matrix_new_f32(const float* data, const uint64_t* rows, const uint64_t* cols,
                          uint64_t nnz, uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                          uint64_t* indices_out, float* data_out, or_err* err) {
  return csr_matrix_new<float>(data, rows, cols, nnz, nrows, ncols, indptr_out, indices_out,
                               data_out, err);
}
int or_csr_matrix_from_raw_check(const uint64_t* indptr, uint64_t indptr_len,
                                 const uint64_t* indices, uint64_t indices_len, uint64_t data_len,
                                 uint64_t nrows, uint64_t ncols, or_err* err) {
  return csr_matrix_from_raw_check(indptr, indptr_len, indices, indices_len, data_len, nrows,
                                   ncols, err);
}
int or_csr_array_new_check(const uint64_t* indptr, uint64_t indptr_len, const uint64_t* indices,
                           uint64_t indices_len, uint64_t data_len, uint64_t nrows,
                           uint64_t ncols, int* has_sorted_indices, or_err* err) {
  return csr_array_new_check(indptr, indptr_len, indices, indices_len, data_len, nrows, ncols,
                             has_sorted_indices, err);
}
int or_csr_array_from_triplets_f64(const uint64_t* rows, const uint64_t* cols,
                                   const double* data, uint64_t nnz, uint64_t nrows,
                                   uint64_t ncols, int sorted, uint64_t* indptr_out,
                                   uint64_t* indices_out, double* data_out,
                                   int* has_sorted_indices, or_err* err) {
  return csr_array_from_triplets<double>(rows, cols, data, nnz, nrows, ncols, sorted, indptr_out,
                                         indices_out, data_out, has_sorted_indices, err);
}
int or_csr_array_from_triplets_f32(const uint64_t* rows, const uint64_t* cols, const float* data,
                                   uint64_t nnz, uint64_t nrows, uint64_t ncols, int sorted,
                                   uint64_t* indptr_out, uint64_t* indices_out, float* data_out,
                                   int* has_sorted_indices, or_err* err) {
  return csr_array_from_triplets<float>(rows, cols, data, nnz, nrows, ncols, sorted, indptr_out,
                                        indices_out, data_out, has_sorted_indices, err);
}
void or_csr_transpose_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                          uint64_t nrows, uint64_t ncols, uint64_t* indptr_t,
                          uint64_t* indices_t, double* data_t) {
  csr_transpose<double>(indptr, indices, data, nrows, ncols, indptr_t, indices_t, data_t);
}
void or_csr_transpose_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                          uint64_t nrows, uint64_t ncols, uint64_t* indptr_t,
                          uint64_t* indices_t, float* data_t) {
  csr_transpose<float>(indptr, indices, data, nrows, ncols, indptr_t, indices_t, data_t);
}
double or_csr_get_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                      uint64_t nrows, uint64_t ncols, uint64_t i, uint64_t j) {
  return csr_get<double>(indptr, indices, data, nrows, ncols, i, j);
}
void or_spmv_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                 uint64_t nrows, const double* x, double* y) {
  spmv<double>(indptr, indices, data, nrows, x, y);
}
void or_spmv_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                 uint64_t nrows, const float* x, float* y) {
  spmv<float>(indptr, indices, data, nrows, x, y);
}
void or_spmv_i32_f64(const int64_t* indptr, const int32_t* indices, const double* data,
                     int64_t nrows, const double* x, double* y) {
  spmv<double>(indptr, indices, data, (uint64_t)nrows, x, y);
}
void or_spmv_i32_f32(const int64_t* indptr, const int32_t* indices, const float* data,
                     int64_t nrows, const float* x, float* y) {
  spmv<float>(indptr, indices, data, (uint64_t)nrows, x, y);
}

or_op* or_op_csr(int f64, const uint64_t* indptr, const uint64_t* indices, const void* data,
                 uint64_t nrows, uint64_t ncols) {
  auto* op = new CsrOp();
  op->f64 = f64; op->nrows = nrows; op->ncols = ncols;
  op->indptr.assign(indptr, indptr + nrows + 1);
  uint64_t nnz = indptr[nrows];
  op->indices.assign(indices, indices + nnz);
  if (f64) {
    const double* d = (const double*)data;
    op->d64.assign(d, d + nnz);
    op->d32.resize(nnz);
    for (uint64_t k = 0; k < nnz; ++k) op->d32[k] = (float)d[k];
  } else {
    const float* d = (const float*)data;
    op->d32.assign(d, d + nnz);
    op->d64.resize(nnz);
    for (uint64_t k = 0; k < nnz; ++k) op->d64[k] = (double)d[k];
  }
  return op;
}
or_op* or_op_csr_i32(int f64, const int64_t* indptr, const int32_t* indices, const void* data,
                     int64_t nrows, int64_t ncols) {
  std::vector<uint64_t> p(nrows + 1), ix(indptr[nrows]);
  for (int64_t i = 0; i <= nrows; ++i) p[i] = (uint64_t)indptr[i];
  for (int64_t k = 0; k < indptr[nrows]; ++k) ix[k] = (uint64_t)indices[k];
  return or_op_csr(f64, p.data(), ix.data(), data, nrows, ncols);
}
or_op* or_op_identity(int f64, uint64_t n) {
  auto* op = new IdentityOp();
  op->f64 = f64; op->nrows = op->ncols = n;
  return op;
}
or_op* or_op_scaled_identity(int f64, uint64_t n, double scale) {
  auto* op = new ScaledIdentityOp();
  op->f64 = f64; op->nrows = op->ncols = n;
  op->s64 = scale; op->s32 = (float)scale;
  return op;
}
or_op* or_op_diagonal(int f64, const void* diag, uint64_t n) {
  auto* op = new DiagOp();
  op->f64 = f64; op->nrows = op->ncols = n;
  op->d64.resize(n); op->d32.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (f64) { op->d64[i] = ((const double*)diag)[i]; op->d32[i] = (float)op->d64[i]; }
    else { op->d32[i] = ((const float*)diag)[i]; op->d64[i] = op->d32[i]; }
  }
  return op;
}

// JacobiPreconditioner::new / from_diagonal, preconditioners.rs:21-62
or_op* or_op_jacobi(const or_op* csr_base, or_err* err) {
  const CsrOp* a = dynamic_cast<const CsrOp*>(csr_base);
  if (!a) { set_err(err, E_NOT_SUPPORTED, "Operation not supported: not a CSR operator"); return nullptr; }
  auto* op = new DiagOp();
  op->f64 = a->f64; op->nrows = op->ncols = a->nrows;
  op->d64.resize(a->nrows); op->d32.resize(a->nrows);
  for (uint64_t i = 0; i < a->nrows; ++i) {
    if (a->f64) {
      double d = csr_get<double>(a->indptr.data(), a->indices.data(), a->d64.data(), a->nrows,
                                 a->ncols, i, i);
      if (std::fabs(d) < std::numeric_limits<double>::epsilon()) {
        delete op;
        set_err(err, E_VALUE, value_msg("Zero diagonal element at position " + std::to_string(i)));
        return nullptr;
      }
      op->d64[i] = 1.0 / d;
      op->d32[i] = (float)op->d64[i];
    } else {
      float d = csr_get<float>(a->indptr.data(), a->indices.data(), a->d32.data(), a->nrows,
                               a->ncols, i, i);
      if (std::fabs(d) < std::numeric_limits<float>::epsilon()) {
        delete op;
        set_err(err, E_VALUE, value_msg("Zero diagonal element at position " + std::to_string(i)));
        return nullptr;
      }
      op->d32[i] = 1.0f / d;
      op->d64[i] = op->d32[i];
    }
  }
  ok(err);
  return op;
}
or_op* or_op_ilu0(const or_op* csr_base, or_err* err) {
  const CsrOp* a = dynamic_cast<const CsrOp*>(csr_base);
  if (!a) { set_err(err, E_NOT_SUPPORTED, "Operation not supported: not a CSR operator"); return nullptr; }
  auto* op = new ILU0Op();
  op->f64 = a->f64; op->nrows = op->ncols = a->nrows;
  const int rc = a->f64 ? ilu0_factor<double>(a, op->f64d, err) : ilu0_factor<float>(a, op->f32d, err);
  if (rc) { delete op; return nullptr; }
  return op;
}

or_op* or_op_ssor(const or_op* csr_base, double omega, or_err* err) {
  const CsrOp* a = dynamic_cast<const CsrOp*>(csr_base);
  if (!a) { set_err(err, E_NOT_SUPPORTED, "Operation not supported: not a CSR operator"); return nullptr; }
  const bool bad = a->f64 ? (omega <= 0.0 || omega >= 2.0) : ((float)omega <= 0.0f || (float)omega >= 2.0f);
  if (bad) { set_err(err, E_VALUE, value_msg("Relaxation parameter omega must be in (0, 2)")); return nullptr; }
  auto* op = new SSOROp();
  op->a = a; op->f64 = a->f64; op->nrows = op->ncols = a->nrows;
  op->om64 = omega; op->om32 = (float)omega;
  op->d64.resize(a->nrows); op->d32.resize(a->nrows);
  for (uint64_t i = 0; i < a->nrows; ++i) {
    const double d = csr_get<double>(a->indptr.data(), a->indices.data(), a->d64.data(), a->nrows, a->ncols, i, i);
    const float d32 = csr_get<float>(a->indptr.data(), a->indices.data(), a->d32.data(), a->nrows, a->ncols, i, i);
    const bool zero = a->f64 ? std::fabs(d) < std::numeric_limits<double>::epsilon()
                             : std::fabs(d32) < std::numeric_limits<float>::epsilon();
    if (zero) {
      delete op;
      set_err(err, E_VALUE, value_msg("Zero diagonal element at position " + std::to_string(i)));
      return nullptr;
    }
    op->d64[i] = d;
    op->d32[i] = d32;
  }
  ok(err);
  return op;
}

or_op* or_op_jacobi_from_diagonal(int f64, const void* diag, uint64_t n, or_err* err) {
  auto* op = new DiagOp();
  op->f64 = f64; op->nrows = op->ncols = n;
  op->d64.resize(n); op->d32.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (f64) {
      double d = ((const double*)diag)[i];
      if (std::fabs(d) < std::numeric_limits<double>::epsilon()) {
        delete op;
        set_err(err, E_VALUE, value_msg("Zero diagonal element at position " + std::to_string(i)));
        return nullptr;
      }
      op->d64[i] = 1.0 / d; op->d32[i] = (float)op->d64[i];
    } else {
      float d = ((const float*)diag)[i];
      if (std::fabs(d) < std::numeric_limits<float>::epsilon()) {
        delete op;
        set_err(err, E_VALUE, value_msg("Zero diagonal element at position " + std::to_string(i)));
        return nullptr;
      }
      op->d32[i] = 1.0f / d; op->d64[i] = op->d32[i];
    }
  }
  ok(err);
  return op;
}

or_op* or_op_ic0(const or_op* csr_base, int fast, or_err* err) {
  const CsrOp* a = dynamic_cast<const CsrOp*>(csr_base);
  if (!a) { set_err(err, E_NOT_SUPPORTED, "Operation not supported: not a CSR operator"); return nullptr; }
  auto* op = new IC0Op();
  op->f64 = a->f64; op->nrows = op->ncols = a->nrows; op->fast = fast != 0;
  int rc = a->f64 ? ic0_factor<double>(a, op->l64, err) : ic0_factor<float>(a, op->l32, err);
  if (rc) { delete op; return nullptr; }
  return op;
}

uint64_t or_ic0_nnz(const or_op* base) {
  const IC0Op* op = dynamic_cast<const IC0Op*>(base);
  if (!op) return 0;
  return op->f64 ? op->l64.indices.size() : op->l32.indices.size();
}
void or_ic0_factor(const or_op* base, uint64_t* indptr, uint64_t* indices, void* data) {
  const IC0Op* op = dynamic_cast<const IC0Op*>(base);
  if (!op) return;
  if (op->f64) {
    std::copy(op->l64.indptr.begin(), op->l64.indptr.end(), indptr);
    std::copy(op->l64.indices.begin(), op->l64.indices.end(), indices);
    std::memcpy(data, op->l64.data.data(), op->l64.data.size() * 8);
  } else {
    std::copy(op->l32.indptr.begin(), op->l32.indptr.end(), indptr);
    std::copy(op->l32.indices.begin(), op->l32.indices.end(), indices);
    std::memcpy(data, op->l32.data.data(), op->l32.data.size() * 4);
  }
}

or_op* or_op_fsai(const or_op* g_base) {
  const CsrOp* g = dynamic_cast<const CsrOp*>(g_base);
  if (!g) return nullptr;
  auto* op = new FsaiOp();
  op->f64 = g->f64; op->nrows = op->ncols = g->nrows;
  op->gp = g->indptr; op->gi = g->indices; op->g64 = g->d64; op->g32 = g->d32;
  uint64_t nnz = g->indptr[g->nrows];
  op->tp.resize(g->ncols + 1); op->ti.resize(nnz); op->t64.resize(nnz); op->t32.resize(nnz);
  csr_transpose<double>(g->indptr.data(), g->indices.data(), g->d64.data(), g->nrows, g->ncols,
                        op->tp.data(), op->ti.data(), op->t64.data());
  std::vector<uint64_t> tp2(g->ncols + 1), ti2(nnz);
  csr_transpose<float>(g->indptr.data(), g->indices.data(), g->d32.data(), g->nrows, g->ncols,
                       tp2.data(), ti2.data(), op->t32.data());
  return op;
}

void or_op_destroy(or_op* op) { delete op; }
uint64_t or_op_rows(const or_op* op) { return op->nrows; }
int or_op_matvec(const or_op* op, const void* x, void* y) {
  if (op->f64) op->mv64((const double*)x, (double*)y);
  else op->mv32((const float*)x, (float*)y);
  return 0;
}

int or_cg(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
          const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err) {
  if (int rc = check_square_and_len<double>(a, "CG", err)) return rc;
  const uint64_t n = a->nrows;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    auto s = cg<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m);
    fill_result(s, x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    auto s = cg<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m);
    fill_result(s, x_out, res);
  }
  return ok(err);
}

int or_bicgstab(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
                const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
                or_err* err) {
  if (int rc = check_square_and_len<double>(a, "BiCGSTAB", err)) return rc;
  const uint64_t n = a->nrows;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    auto s = bicgstab<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m1, m2);
    fill_result(s, x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    auto s = bicgstab<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m1, m2);
    fill_result(s, x_out, res);
  }
  return ok(err);
}

int or_gmres(const or_op* a, const void* b, uint64_t max_iter, uint64_t restart, double rtol,
             double atol, const void* x0, const or_op* m, void* x_out, or_result* res,
             or_err* err) {
  if (int rc = check_square_and_len<double>(a, "GMRES", err)) return rc;
  const uint64_t n = a->nrows;
  int stalled = 0;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    auto s = gmres<double>(a, bv, max_iter, restart, rtol, atol, (const double*)x0, m);
    fill_result(s, x_out, res);
    stalled = s.stalled;
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    auto s = gmres<float>(a, bv, max_iter, restart, (float)rtol, (float)atol, (const float*)x0, m);
    fill_result(s, x_out, res);
    stalled = s.stalled;
  }
  if (stalled)
    return restart == 0
               ? set_err(err, E_VALUE, value_msg("restart = 0 makes no progress (the reference loops forever)"))
               : set_err(err, E_COMPUTATION,
                         "Computation error: gmres cannot advance: breakdown at the first Arnoldi step "
                         "(the reference loops forever)");
  return ok(err);
}


int or_bicg(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
            const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
            or_err* err) {
  if (int rc = check_square_and_len<double>(a, "BiCG", err)) return rc;
  const uint64_t n = a->nrows;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    fill_result(bicg<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m1, m2), x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    fill_result(bicg<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m1, m2), x_out, res);
  }
  return ok(err);
}

int or_cgs(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
           const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err) {
  if (int rc = check_square_and_len<double>(a, "CGS", err)) return rc;
  const uint64_t n = a->nrows;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    fill_result(cgs<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m), x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    fill_result(cgs<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m), x_out, res);
  }
  return ok(err);
}

int or_qmr(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
           const void* x0, const or_op* m1, const or_op* m2, void* x_out, or_result* res,
           or_err* err) {
  // qmr.rs:53-59: DimensionMismatch{expected: b.len(), found: rows}
  const uint64_t n = a->nrows;
  if (a->ncols != n)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(n, a->nrows), n, a->nrows);
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    fill_result(qmr<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m1, m2), x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    fill_result(qmr<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m1, m2), x_out, res);
  }
  return ok(err);
}

int or_minres(const or_op* a, const void* b, uint64_t max_iter, double rtol, double atol,
              const void* x0, const or_op* m, void* x_out, or_result* res, or_err* err) {
  if (a->nrows != a->ncols)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(a->nrows, a->ncols), a->nrows, a->ncols);
  const uint64_t n = a->nrows;
  int e = 0;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    auto s = minres<double>(a, bv, max_iter, rtol, atol, (const double*)x0, m, &e);
    if (!e) fill_result(s, x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    auto s = minres<float>(a, bv, max_iter, (float)rtol, (float)atol, (const float*)x0, m, &e);
    if (!e) fill_result(s, x_out, res);
  }
  if (e == 1) return set_err(err, E_COMPUTATION, "Computation error: Indefinite preconditioner");
  if (e == 2) return set_err(err, E_COMPUTATION, "Computation error: Non-symmetric matrix");
  return ok(err);
}

int or_lgmres(const or_op* a, const void* b, uint64_t max_iter, uint64_t inner_m, double rtol,
              double atol, const void* x0, const or_op* m, void* x_out, or_result* res,
              or_err* err) {
  if (a->nrows != a->ncols)
    return set_err(err, E_DIMENSION_MISMATCH, dim_msg(a->nrows, a->ncols), a->nrows, a->ncols);
  const uint64_t n = a->nrows;
  if (a->f64) {
    std::vector<double> bv((const double*)b, (const double*)b + n);
    fill_result(lgmres<double>(a, bv, max_iter, inner_m, rtol, atol, (const double*)x0, m), x_out, res);
  } else {
    std::vector<float> bv((const float*)b, (const float*)b + n);
    fill_result(lgmres<float>(a, bv, max_iter, inner_m, (float)rtol, (float)atol, (const float*)x0, m), x_out,
                res);
  }
  return ok(err);
}

double or_true_rel_residual(const int64_t* indptr, const int32_t* indices, const double* data,
                            int64_t n, const double* b, const double* x) {
  std::vector<double> ax(n);
  spmv<double>(indptr, indices, data, (uint64_t)n, x, ax.data());
  double rr = 0, bb = 0;
  for (int64_t i = 0; i < n; ++i) {
    double r = b[i] - ax[i];
    rr = rr + r * r;
    bb = bb + b[i] * b[i];
  }
  return std::sqrt(rr) / std::sqrt(bb);
}

// FP64 iterative refinement around an FP32 Jacobi-PCG (the algorithm of the
// device's mixed-precision solver; no reference counterpart):
//   x = 0; repeat: r = b - A x (FP64); stop if ||r|| <= tol ||b||;
//   d = cg_f32(A32, r / ||r||); x += ||r|| * d.
int or_cg_mixed_ir(const int64_t* indptr, const int32_t* indices, const double* data, int64_t n,
                   const double* b, const or_ir_options* opt, double* x, or_ir_result* res) {
  or_op* a32 = or_op_csr_i32(1, indptr, indices, data, n, n);
  // the inner operator works on the FP32 copy of the values
  a32->f64 = 0;
  or_op* m = nullptr;
  if (opt->jacobi) {
    or_err e;
    m = or_op_jacobi(a32, &e);
    if (!m) { delete a32; return 1; }
  }
  std::vector<double> xv(n, 0.0), r(n), ax(n);
  double bb = 0;
  for (int64_t i = 0; i < n; ++i) bb = bb + b[i] * b[i];
  const double bnorm = std::sqrt(bb);
  uint64_t outer = 0, inner_total = 0;
  double rel = 0;
  bool conv = false;
  while (true) {
    spmv<double>(indptr, indices, data, (uint64_t)n, xv.data(), ax.data());
    double rr = 0;
    for (int64_t i = 0; i < n; ++i) { r[i] = b[i] - ax[i]; rr = rr + r[i] * r[i]; }
    double rnorm = std::sqrt(rr);
    rel = rnorm / bnorm;
    if (rnorm <= opt->tol * bnorm) { conv = true; break; }
    if (outer >= opt->max_outer) break;
    std::vector<float> r32(n);
    for (int64_t i = 0; i < n; ++i) r32[i] = (float)(r[i] / rnorm);
    auto s = cg<float>(a32, r32, opt->max_inner, (float)opt->inner_rtol, 0.0f, nullptr, m);
    inner_total += s.iterations;
    for (int64_t i = 0; i < n; ++i) xv[i] = xv[i] + rnorm * (double)s.x[i];
    ++outer;
  }
  std::memcpy(x, xv.data(), n * 8);
  if (res) {
    res->outer_iterations = outer;
    res->inner_iterations = inner_total;
    res->rel_residual = rel;
    res->converged = conv ? 1 : 0;
  }
  delete m;
  delete a32;
  return 0;
}

// FP32 PCG with FP64 residual replacement (restates the device loop of
// sx_cg_mixed, mode SX_IR_REPLACE):
//   x64 = 0, r = b (FP64); r32 = (float) r; x32 = 0; z = M r32; p = z;
//   segment: CG iterations on (x32, r32, p) until ||r32|| <= max(atol, delta ||r32_0||)
//            with atol = 0.5 tol ||b|| (FP32), or pAp <= 0, or max_inner;
//   then x64 += x32, x32 = 0, r = b - A x64 (FP64); stop if ||r|| <= tol ||b||;
//   r32 = (float) r; z = M r32; beta = r32.z / rz_old; p = z + beta p; next segment.
//   Stops unconverged after max_outer replacements or two replacements in a
//   row that fail to halve the FP64 residual.
int or_cg_mixed_replace(const int64_t* indptr, const int32_t* indices, const double* data, int64_t n,
                        const double* b, const or_ir_options* opt, double delta, double* x,
                        or_ir_result* res) {
  or_op* a32 = or_op_csr_i32(1, indptr, indices, data, n, n);
  a32->f64 = 0;
  or_op* m = nullptr;
  if (opt->jacobi) {
    or_err e;
    m = or_op_jacobi(a32, &e);
    if (!m) { delete a32; return 1; }
  }
  std::vector<double> x64(n, 0.0), r64(n), ax(n);
  auto true_residual = [&]() {
    spmv<double>(indptr, indices, data, (uint64_t)n, x64.data(), ax.data());
    double rr = 0;
    for (int64_t i = 0; i < n; ++i) { r64[i] = b[i] - ax[i]; rr = rr + r64[i] * r64[i]; }
    return std::sqrt(rr);
  };
  double bb = 0;
  for (int64_t i = 0; i < n; ++i) bb = bb + b[i] * b[i];
  const double bnorm = std::sqrt(bb);
  double rnorm = true_residual();
  double rel = rnorm / bnorm;
  uint64_t outer = 0, inner = 0;
  bool conv = rnorm <= opt->tol * bnorm;
  if (!conv) {
    std::vector<float> r(n), x32(n, 0.0f), z, p, ap;
    for (int64_t i = 0; i < n; ++i) r[i] = (float)r64[i];
    z = m ? op_apply(m, r) : r;
    p = z;
    float rz_old = dot(r, z);
    const float atol = (float)(0.5 * opt->tol * bnorm);
    float tol = std::fmax(atol, (float)delta * norm2(r));
    double prev = rnorm;
    int stalls = 0;
    for (;;) {
      bool not_pd = false;
      for (uint64_t it = 0; it < opt->max_inner; ++it) {
        ap = op_apply(a32, p);
        const float pap = dot(p, ap);
        if (pap <= 0.0f) { not_pd = true; break; }
        const float alpha = rz_old / pap;
        for (int64_t i = 0; i < n; ++i) x32[i] += alpha * p[i];
        for (int64_t i = 0; i < n; ++i) r[i] -= alpha * ap[i];
        ++inner;
        if (norm2(r) <= tol) break;
        z = m ? op_apply(m, r) : r;
        const float rz_new = dot(r, z);
        const float beta = rz_new / rz_old;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz_old = rz_new;
      }
      for (int64_t i = 0; i < n; ++i) { x64[i] = x64[i] + (double)x32[i]; x32[i] = 0.0f; }
      rnorm = true_residual();
      rel = rnorm / bnorm;
      ++outer;
      if (rnorm <= opt->tol * bnorm) { conv = true; break; }
      if (not_pd || outer >= opt->max_outer) break;
      if (!(rnorm < 0.5 * prev)) {
        if (++stalls >= 2) break;
      } else {
        stalls = 0;
      }
      prev = rnorm;
      for (int64_t i = 0; i < n; ++i) r[i] = (float)r64[i];
      z = m ? op_apply(m, r) : r;
      const float rz = dot(r, z);
      const float beta = rz / rz_old;
      rz_old = rz;
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
      tol = std::fmax(atol, (float)delta * norm2(r));
    }
  }
  std::memcpy(x, x64.data(), n * 8);
  if (res) {
    res->outer_iterations = outer;
    res->inner_iterations = inner;
    res->rel_residual = rel;
    res->converged = conv ? 1 : 0;
  }
  delete m;
  delete a32;
  return 0;
}

}  // extern "C"

// ------------------------------------------------ symmetric CSR (lower part)
namespace {

// SymCsrMatrix::new checks, sym_csr.rs:70-126, in that order.
int sym_check(uint64_t data_len, const uint64_t* indptr, uint64_t indptr_len,
              const uint64_t* indices, uint64_t nnz, uint64_t rows, uint64_t cols, or_err* err) {
  if (rows != cols) return set_err(err, E_VALUE, value_msg("Symmetric matrix must be square"));
  if (indptr_len != rows + 1)
    return set_err(err, E_VALUE,
                   value_msg("indptr length (" + std::to_string(indptr_len) +
                             ") must be equal to rows + 1 (" + std::to_string(rows + 1) + ")"));
  if (data_len != nnz)
    return set_err(err, E_VALUE,
                   value_msg("data length (" + std::to_string(data_len) +
                             ") must match indices length (" + std::to_string(nnz) + ")"));
  if (indptr[rows] != nnz)
    return set_err(err, E_VALUE,
                   value_msg("Last indptr value (" + std::to_string(indptr[rows]) +
                             ") must equal nnz (" + std::to_string(nnz) + ")"));
  for (uint64_t i = 0; i < rows; ++i) {
    if (indptr[i] > indptr[i + 1] || indptr[i + 1] > nnz)
      return set_err(err, E_INCONSISTENT_DATA, incons_msg("row pointers must be non-decreasing"));
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      const uint64_t c = indices[k];
      if (c >= cols)
        return set_err(err, E_INDEX_OUT_OF_BOUNDS,
                       "Index (" + std::to_string(i) + ", " + std::to_string(c) +
                           ") out of bounds for array with shape (" + std::to_string(rows) + ", " +
                           std::to_string(cols) + ")",
                       i, c, rows, cols);
      if (c > i)
        return set_err(err, E_VALUE,
                       value_msg("Symmetric CSR should only store the lower triangular part"));
    }
  }
  return ok(err);
}

// sym_csr_matvec, sym_ops.rs:69-87: y = 0; for each stored (i, j, v) in row
// order: y_i = y_i + v x_j and, when i != j, y_j = y_j + v x_i.
template <class T>
void sym_matvec(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t n,
                const T* x, T* y) {
  for (uint64_t i = 0; i < n; ++i) y[i] = T(0);
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      const uint64_t c = indices[k];
      const T v = data[k];
      y[i] = y[i] + v * x[c];
      if (i != c) y[c] = y[c] + v * x[i];
    }
}

// sym_csr_trace, sym_ops.rs:321-334: the first diagonal entry of each row.
template <class T>
T sym_trace(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t n) {
  T t = T(0);
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k)
      if (indices[k] == i) {
        t = t + data[k];
        break;
      }
  return t;
}

// sym_csr_quadratic_form, sym_ops.rs:275-282.
template <class T>
T sym_quad(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t n, const T* x) {
  std::vector<T> ax(n);
  sym_matvec<T>(indptr, indices, data, n, x, ax.data());
  T r = T(0);
  for (uint64_t i = 0; i < n; ++i) r = r + x[i] * ax[i];
  return r;
}

// sym_csr_rank1_update, sym_ops.rs:199-231: dense lower triangle (stored
// entries, the last duplicate wins), + alpha x_i x_j, non-zeros kept.
template <class T>
uint64_t sym_rank1(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t n,
                   const T* x, T alpha, uint64_t* ip, uint64_t* ix, T* dv) {
  std::vector<T> row(n);
  uint64_t cnt = 0;
  if (ip) ip[0] = 0;
  for (uint64_t i = 0; i < n; ++i) {
    std::fill(row.begin(), row.end(), T(0));
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k) row[indices[k]] = data[k];
    for (uint64_t j = 0; j <= i; ++j) {
      const T update = alpha * x[i] * x[j];
      const T v = row[j] + update;
      if (v != T(0)) {
        if (ix) {
          ix[cnt] = j;
          dv[cnt] = v;
        }
        ++cnt;
      }
    }
    if (ip) ip[i + 1] = cnt;
  }
  return cnt;
}

// SymCsrMatrix::from_csr, sym_csr.rs:149-189, with is_symmetric (:197-225)
// reading CsrMatrix::get's first match.
template <class T>
int sym_from_csr(const uint64_t* indptr, const uint64_t* indices, const T* data, uint64_t rows,
                 uint64_t cols, uint64_t* ip, uint64_t* ix, T* dv, or_err* err) {
  if (rows != cols) return set_err(err, E_VALUE, value_msg("Symmetric matrix must be square"));
  const T tol = std::numeric_limits<T>::epsilon() * T(100.0);
  for (uint64_t i = 0; i < rows; ++i)
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      const uint64_t j = indices[k];
      const T other = csr_get<T>(indptr, indices, data, rows, cols, j, i);
      const T diff = std::fabs(data[k] - other);
      if (diff > tol)
        return set_err(err, E_VALUE,
                       value_msg("Matrix must be symmetric to convert to SymCSR format"));
    }
  uint64_t cnt = 0;
  ip[0] = 0;
  for (uint64_t i = 0; i < rows; ++i) {
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k)
      if (indices[k] <= i) {
        ix[cnt] = indices[k];
        dv[cnt] = data[k];
        ++cnt;
      }
    ip[i + 1] = cnt;
  }
  return ok(err);
}

}  // namespace

extern "C" {

int or_sym_csr_check(uint64_t data_len, const uint64_t* indptr, uint64_t indptr_len,
                     const uint64_t* indices, uint64_t nnz, uint64_t nrows, uint64_t ncols,
                     or_err* err) {
  return sym_check(data_len, indptr, indptr_len, indices, nnz, nrows, ncols, err);
}
void or_sym_csr_matvec_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                           uint64_t n, const double* x, double* y) {
  sym_matvec<double>(indptr, indices, data, n, x, y);
}
void or_sym_csr_matvec_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                           uint64_t n, const float* x, float* y) {
  sym_matvec<float>(indptr, indices, data, n, x, y);
}
uint64_t or_sym_csr_nnz(const uint64_t* indptr, const uint64_t* indices, uint64_t nnz_stored,
                        uint64_t n) {
  // sym_csr.rs:254-268
  uint64_t diag = 0;
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t k = indptr[i]; k < indptr[i + 1]; ++k)
      if (indices[k] == i) {
        ++diag;
        break;
      }
  return diag + 2 * (nnz_stored - diag);
}
double or_sym_csr_get_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                          uint64_t n, uint64_t row, uint64_t col) {
  // sym_csr.rs:280-298
  if (row >= n || col >= n) return 0.0;
  const uint64_t r = row < col ? col : row, c = row < col ? row : col;
  for (uint64_t k = indptr[r]; k < indptr[r + 1]; ++k)
    if (indices[k] == c) return data[k];
  return 0.0;
}
double or_sym_csr_trace_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                            uint64_t n) {
  return sym_trace<double>(indptr, indices, data, n);
}
float or_sym_csr_trace_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                           uint64_t n) {
  return sym_trace<float>(indptr, indices, data, n);
}
double or_sym_csr_quadratic_form_f64(const uint64_t* indptr, const uint64_t* indices,
                                     const double* data, uint64_t n, const double* x) {
  return sym_quad<double>(indptr, indices, data, n, x);
}
float or_sym_csr_quadratic_form_f32(const uint64_t* indptr, const uint64_t* indices,
                                    const float* data, uint64_t n, const float* x) {
  return sym_quad<float>(indptr, indices, data, n, x);
}
uint64_t or_sym_csr_rank1_update_f64(const uint64_t* indptr, const uint64_t* indices,
                                     const double* data, uint64_t n, const double* x,
                                     double alpha, uint64_t* indptr_out, uint64_t* indices_out,
                                     double* data_out) {
  return sym_rank1<double>(indptr, indices, data, n, x, alpha, indptr_out, indices_out, data_out);
}
uint64_t or_sym_csr_rank1_update_f32(const uint64_t* indptr, const uint64_t* indices,
                                     const float* data, uint64_t n, const float* x, float alpha,
                                     uint64_t* indptr_out, uint64_t* indices_out,
                                     float* data_out) {
  return sym_rank1<float>(indptr, indices, data, n, x, alpha, indptr_out, indices_out, data_out);
}
int or_sym_csr_from_csr_f64(const uint64_t* indptr, const uint64_t* indices, const double* data,
                            uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                            uint64_t* indices_out, double* data_out, or_err* err) {
  return sym_from_csr<double>(indptr, indices, data, nrows, ncols, indptr_out, indices_out,
                              data_out, err);
}
int or_sym_csr_from_csr_f32(const uint64_t* indptr, const uint64_t* indices, const float* data,
                            uint64_t nrows, uint64_t ncols, uint64_t* indptr_out,
                            uint64_t* indices_out, float* data_out, or_err* err) {
  return sym_from_csr<float>(indptr, indices, data, nrows, ncols, indptr_out, indices_out,
                             data_out, err);
}

}  // extern "C"

// ------------------------------------------------------------------ eigen
// scirs2-sparse/src/linalg/eigen.rs: power_iteration (:124-293), lanczos
// (:295-494) and their tridiagonal helpers (:512-936), restated with the
// reference's arithmetic order and its quirks:
//   - lanczos never updates beta_j after the first step (the update at
//     :441-443 binds a new variable that dies at once), so every Lanczos
//     vector is w / beta_1 and every off-diagonal entry is beta_1;
//   - the QL sweep (:551-632) leaves its loop after one sweep for l >= 1
//     (the `i < l` test at :617 fires whenever the sweep runs to its end);
//   - Ritz vectors and the Kaniel-Paige bound index the eigenvector list as
//     eigvecs[j][k] (:459, :485), i.e. the transpose of the list returned;
//   - where the reference would panic (an index past the end of a list, a
//     subspace of size 0) the restatement returns a ComputationError that
//     names the panic.
namespace {

template <class T>
T fold_dot(const std::vector<T>& a, const std::vector<T>& b) {
  T s = T(0);
  for (size_t i = 0; i < a.size(); ++i) s = s + a[i] * b[i];
  return s;
}

// solve_cubic, eigen.rs:890-952
template <class T>
std::vector<T> solve_cubic(T p, T q, T r) {
  const T p3 = p / T(3.0);
  const T p3sq = p3 * p3;
  const T a = q - p * p3;
  const T b = r + p3 * (T(2.0) * p3sq - q);
  const T disc = T(4.0) * a * a * a + T(27.0) * b * b;
  std::vector<T> roots;
  if (disc == T(0)) {
    if (a == T(0)) {
      roots.assign(3, -p3);
    } else {
      const T x1 = T(3.0) * b / a;
      const T x2 = -x1 / T(2.0);
      roots = {x1 - p3, x2 - p3, x2 - p3};
    }
  } else if (disc > T(0)) {
    const T sd = std::sqrt(disc);
    const T c1 = (-b + sd * T(0.5)) / T(2.0);
    const T c2 = (-b - sd * T(0.5)) / T(2.0);
    const T third = (T)(1.0 / 3.0);
    const T c1r = std::pow(std::fabs(c1), third) * (c1 >= T(0) ? T(1) : T(-1));
    const T c2r = std::pow(std::fabs(c2), third) * (c2 >= T(0) ? T(1) : T(-1));
    roots.push_back(c1r + c2r - p3);
  } else {
    const T ps = std::sqrt(-a / T(3.0));
    const T theta = std::acos(b / (T(2.0) * ps * ps * ps));
    for (int k = 0; k < 3; ++k) {
      const T ang = (T)(3.141592653589793 * (2.0 * (double)k) / 3.0);
      roots.push_back(T(2.0) * ps * std::cos(ang - theta / T(3.0)) - p3);
    }
  }
  return roots;
}

// descending order of partial_cmp with incomparable pairs Equal (a stable
// sort, as Rust's sort_by)
template <class T>
bool desc_less(T x, T y) { return x > y; }

const char* kPanicIndex = "panic: index out of bounds in the reference's eigenvector lists";

// solve_small_tridiagonal, eigen.rs:650-886
template <class T>
int small_tridiag(const std::vector<T>& alpha, const std::vector<T>& beta, size_t num, std::vector<T>& vals,
                  std::vector<std::vector<T>>& vecs, or_err* err) {
  const size_t n = alpha.size();
  vals.clear();
  vecs.clear();
  if (n == 1) {
    vals = {alpha[0]};
    vecs = {{T(1)}};
    return ok(err);
  }
  if (n == 2) {
    const T a = alpha[0], b = alpha[1], c = beta[0];
    const T trace = a + b;
    const T det = a * b - c * c;
    const T disc = std::sqrt(trace * trace - T(4.0) * det);
    T l1 = (trace + disc) * T(0.5), l2 = (trace - disc) * T(0.5);
    if (!(l1 >= l2)) std::swap(l1, l2);
    std::vector<T> v1(2, T(0)), v2(2, T(0));
    if (c != T(0)) {
      v1[0] = c; v1[1] = l1 - a;
      v2[0] = c; v2[1] = l2 - a;
      const T n1 = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1]);
      const T n2 = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1]);
      if (n1 != T(0)) { v1[0] = v1[0] / n1; v1[1] = v1[1] / n1; }
      if (n2 != T(0)) { v2[0] = v2[0] / n2; v2[1] = v2[1] / n2; }
    } else if (a >= b) {
      v1 = {T(1), T(0)}; v2 = {T(0), T(1)};
    } else {
      v1 = {T(0), T(1)}; v2 = {T(1), T(0)};
    }
    vals = {l1, l2};
    vecs = {v1, v2};
    if (vals.size() > num) vals.resize(num);
    if (vecs.size() > num) vecs.resize(num);
    return ok(err);
  }
  // n == 3: characteristic polynomial and Vieta's roots
  const T a = alpha[0], b = alpha[1], c = alpha[2], d = beta[0], e = beta[1];
  const T p = -(a + b + c);
  const T q = a * b + a * c + b * c - d * d - e * e;
  const T r = -(a * b * c - a * e * e - c * d * d);
  std::vector<T> sorted = solve_cubic<T>(p, q, r);
  std::stable_sort(sorted.begin(), sorted.end(), desc_less<T>);
  const size_t take = std::min<size_t>(num, 3);
  if (take > sorted.size()) return set_err(err, E_COMPUTATION, "panic: slice index out of range for the cubic's roots");
  for (size_t t = 0; t < take; ++t) {
    const T lambda = sorted[t];
    T m00 = a - lambda, m01 = d, m02 = T(0);
    T m10 = d, m11 = b - lambda, m12 = e;
    T m20 = T(0), m21 = e, m22 = c - lambda;
    const T r0 = std::sqrt(m00 * m00 + m01 * m01 + m02 * m02);
    const T r1 = std::sqrt(m10 * m10 + m11 * m11 + m12 * m12);
    const T r2 = std::sqrt(m20 * m20 + m21 * m21 + m22 * m22);
    std::vector<T> v(3, T(0));
    if (r0 >= r1 && r0 >= r2 && r0 != T(0)) {
      const T s = T(1) / r0;
      m00 = m00 * s; m01 = m01 * s; m02 = m02 * s;
      T f = m10 / m00;
      m11 = m11 - f * m01; m12 = m12 - f * m02;
      f = m20 / m00;
      m21 = m21 - f * m01; m22 = m22 - f * m02;
      v[2] = T(1);
      v[1] = -m12 * v[2] / m11;
      v[0] = -(m01 * v[1] + m02 * v[2]) / m00;
    } else if (r1 >= r0 && r1 >= r2 && r1 != T(0)) {
      const T s = T(1) / r1;
      m10 = m10 * s; m11 = m11 * s; m12 = m12 * s;
      T f = m01 / m11;
      m00 = m00 - f * m10; m02 = m02 - f * m12;
      f = m21 / m11;
      m20 = m20 - f * m10; m22 = m22 - f * m12;
      v[2] = T(1);
      v[0] = -m02 * v[2] / m00;
      v[1] = -(m10 * v[0] + m12 * v[2]) / m11;
    } else if (r2 != T(0)) {
      const T s = T(1) / r2;
      m20 = m20 * s; m21 = m21 * s; m22 = m22 * s;
      T f = m02 / m22;
      m00 = m00 - f * m20; m01 = m01 - f * m21;
      f = m12 / m22;
      m10 = m10 - f * m20; m11 = m11 - f * m21;
      v[0] = T(1);
      v[1] = -m10 * v[0] / m11;
      v[2] = -(m20 * v[0] + m21 * v[1]) / m22;
    } else {
      if (num >= 1) v[0] = T(1);
      else if (num >= 2) v[1] = T(1);
      else v[2] = T(1);
    }
    const T nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (nv != T(0)) { v[0] = v[0] / nv; v[1] = v[1] / nv; v[2] = v[2] / nv; }
    vecs.push_back(v);
  }
  if (sorted.size() > num) sorted.resize(num);
  vals = sorted;
  return ok(err);
}

// solve_tridiagonal_eigenproblem, eigen.rs:512-646
template <class T>
int tridiag_eig(const std::vector<T>& alpha, const std::vector<T>& beta, size_t num, std::vector<T>& vals,
                std::vector<std::vector<T>>& vecs, or_err* err) {
  const size_t n = alpha.size();
  if (n == 0) return set_err(err, E_VALUE, value_msg("Empty tridiagonal matrix"));
  if (beta.size() != n - 1) return set_err(err, E_DIMENSION_MISMATCH, dim_msg(n - 1, beta.size()), n - 1, beta.size());
  if (n <= 3) return small_tridiag<T>(alpha, beta, num, vals, vecs, err);
  std::vector<T> d = alpha, e = beta;
  e.push_back(T(0));
  std::vector<std::vector<T>> z(n, std::vector<T>(n, T(0)));
  for (size_t i = 0; i < n; ++i) z[i][i] = T(1);
  const T small = (T)1e-12;
  for (size_t l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      size_t m = l;
      while (m < n - 1) {
        if (std::fabs(e[m]) <= small * (std::fabs(d[m]) + std::fabs(d[m + 1]))) break;
        ++m;
      }
      if (m == l) break;
      if (iter >= 30) return set_err(err, E_SOLVER_FAILURE, "Iterative solver failure: QL algorithm did not converge");
      T g = (d[l + 1] - d[l]) * T(0.5) / e[l];
      const T r = std::sqrt(g * g + T(1));
      g = d[m] - d[l] + e[l] / (g + (g >= T(0) ? r : -r));
      T s = T(1), c = T(1), p = T(0);
      size_t i = m - 1;
      while (i >= l && i < n) {
        const T f = s * e[i];
        const T b = c * e[i];
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
          const T t = z[k][i + 1];
          z[k][i + 1] = s * z[k][i] + c * t;
          z[k][i] = c * z[k][i] - s * t;
        }
        if (i == 0) break;
        i -= 1;
      }
      if ((int32_t)i < (int32_t)l || i >= n) break;
      if (r == T(0)) {  // unreachable: r >= 1 (kept as written)
        if ((int32_t)m == (int32_t)(l + 1)) break;
        d[l] = d[l] - p;
        e[l] = g;
        e[m - 1] = T(0);
      }
      ++iter;
    }
  }
  std::vector<size_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](size_t i, size_t j) { return d[i] > d[j]; });
  vals.clear();
  vecs.clear();
  for (size_t k = 0; k < std::min(num, n); ++k) {
    vals.push_back(d[idx[k]]);
    std::vector<T> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = z[i][idx[k]];
    vecs.push_back(v);
  }
  return ok(err);
}

struct SymArrays {
  const uint64_t* indptr;
  const uint64_t* indices;
  uint64_t n;
};

// power_iteration, eigen.rs:124-293
template <class T>
int power_iteration(const SymArrays& A, const T* data, uint64_t max_iter, double tol, int normalize, const T* x0,
                    uint64_t x0_len, T* lambda_out, T* vec_out, T* resid_out, or_eig_info* info, or_err* err) {
  const uint64_t n = A.n;
  std::vector<T> x(n, T(0));
  if (x0) {
    if (x0_len != n) return set_err(err, E_DIMENSION_MISMATCH, dim_msg(n, x0_len), n, x0_len);
    for (uint64_t i = 0; i < n; ++i) x[i] = x0[i];
  } else if (n > 0) {
    x[0] = T(1);
  }
  if (normalize) {
    const T nrm = std::sqrt(fold_dot(x, x));
    if (nrm != T(0))
      for (auto& v : x) v = v / nrm;
  }
  const T ttol = (T)tol;
  T lambda = T(0), prev = T(0);
  bool conv = false;
  uint64_t it = 0;
  std::vector<T> y(n);
  while (it < max_iter) {
    sym_matvec<T>(A.indptr, A.indices, data, n, x.data(), y.data());
    const T num = fold_dot(x, y);
    if (normalize) {
      lambda = num;
      if (std::fabs(lambda - prev) < ttol) { conv = true; break; }
      const T nrm = std::sqrt(fold_dot(y, y));
      if (nrm != T(0))
        for (uint64_t i = 0; i < n; ++i) x[i] = y[i] / nrm;
    } else {
      x = y;
      const T nx = std::sqrt(fold_dot(x, x));
      if (nx != T(0)) lambda = num / (nx * nx);
      if (std::fabs(lambda - prev) < ttol) { conv = true; break; }
    }
    prev = lambda;
    ++it;
  }
  sym_matvec<T>(A.indptr, A.indices, data, n, x.data(), y.data());
  T rs = T(0);
  for (uint64_t i = 0; i < n; ++i) {
    const T ri = y[i] - lambda * x[i];
    rs = rs + ri * ri;
  }
  *lambda_out = lambda;
  if (vec_out) for (uint64_t i = 0; i < n; ++i) vec_out[i] = x[i];
  *resid_out = std::sqrt(rs);
  info->iterations = it;
  info->converged = conv ? 1 : 0;
  info->count = 1;
  return ok(err);
}

// lanczos, eigen.rs:295-494
template <class T>
int lanczos(const SymArrays& A, const T* data, uint64_t max_iter, uint64_t max_subspace, double tol,
            uint64_t num_eigenvalues, int compute_vecs, const T* v0, uint64_t v0_len, T* vals_out, T* vecs_out,
            T* resid_out, or_eig_info* info, or_err* err) {
  const uint64_t n = A.n;
  const uint64_t sub = std::min(max_subspace, n);
  const uint64_t num = std::min(num_eigenvalues, sub);
  std::vector<T> v(n, T(0));
  if (v0) {
    if (v0_len != n) return set_err(err, E_DIMENSION_MISMATCH, dim_msg(n, v0_len), n, v0_len);
    for (uint64_t i = 0; i < n; ++i) v[i] = v0[i];
  } else if (n > 0) {
    v[0] = T(1);
  }
  if (sub == 0) return set_err(err, E_COMPUTATION, "panic: capacity overflow (subspace size 0)");
  const T nrm = std::sqrt(fold_dot(v, v));
  if (nrm != T(0))
    for (auto& t : v) t = t / nrm;
  std::vector<std::vector<T>> V{v};
  std::vector<T> alpha, beta;
  std::vector<T> w(n);
  sym_matvec<T>(A.indptr, A.indices, data, n, v.data(), w.data());
  const T a0 = fold_dot(v, w);
  alpha.push_back(a0);
  for (uint64_t i = 0; i < n; ++i) w[i] = w[i] - a0 * v[i];
  const T beta_j = std::sqrt(fold_dot(w, w));  // never updated (see above)
  uint64_t it = 1;
  bool conv = false;
  const T ttol = (T)tol;
  std::vector<T> ev;
  std::vector<std::vector<T>> evec;
  while (it < max_iter && alpha.size() < sub) {
    if (beta_j == T(0)) break;
    beta.push_back(beta_j);
    std::vector<T> vn(n);
    for (uint64_t i = 0; i < n; ++i) vn[i] = w[i] / beta_j;
    V.push_back(vn);
    sym_matvec<T>(A.indptr, A.indices, data, n, vn.data(), w.data());
    for (const auto& vj : V) {
      const T proj = fold_dot(vj, w);
      for (uint64_t i = 0; i < n; ++i) w[i] = w[i] - proj * vj[i];
    }
    const T aj = fold_dot(vn, w);
    alpha.push_back(aj);
    for (uint64_t i = 0; i < n; ++i) w[i] = w[i] - aj * vn[i];
    const T bnext = std::sqrt(fold_dot(w, w));
    if (alpha.size() >= num) {
      int rc = tridiag_eig<T>(alpha, beta, num, ev, evec, err);
      if (rc) return rc;
      if (ev.empty()) return set_err(err, E_COMPUTATION, "panic: index out of bounds (no eigenvalue to test)");
      if (bnext < ttol * std::fabs(ev[0])) { conv = true; break; }
    }
    ++it;
  }
  int rc = tridiag_eig<T>(alpha, beta, num, ev, evec, err);
  if (rc) return rc;
  std::vector<T> ritz;
  if (compute_vecs) {
    ritz.assign(n * num, T(0));
    for (uint64_t k = 0; k < num; ++k)
      for (uint64_t i = 0; i < n; ++i) {
        T s = T(0);
        for (size_t j = 0; j < V.size(); ++j)
          if (j < evec.size()) {
            if (k >= evec[j].size()) return set_err(err, E_COMPUTATION, kPanicIndex);
            s = s + evec[j][k] * V[j][i];
          }
        ritz[i * num + k] = s;
      }
  }
  std::vector<T> res(num, T(0));
  if (compute_vecs) {
    std::vector<T> e(n), ax(n);
    for (uint64_t k = 0; k < num; ++k) {
      if (k >= ev.size()) return set_err(err, E_COMPUTATION, kPanicIndex);
      for (uint64_t i = 0; i < n; ++i) e[i] = ritz[i * num + k];
      sym_matvec<T>(A.indptr, A.indices, data, n, e.data(), ax.data());
      T s = T(0);
      for (uint64_t i = 0; i < n; ++i) {
        const T ri = ax[i] - ev[k] * e[i];
        s = s + ri * ri;
      }
      res[k] = std::sqrt(s);
    }
  } else {
    for (uint64_t k = 0; k < num; ++k)
      if (k < evec.size() && !beta.empty()) {
        if (k >= evec.back().size()) return set_err(err, E_COMPUTATION, kPanicIndex);
        res[k] = beta.back() * std::fabs(evec.back()[k]);
      }
  }
  for (size_t k = 0; k < ev.size(); ++k) vals_out[k] = ev[k];
  for (uint64_t k = 0; k < num; ++k) resid_out[k] = res[k];
  if (compute_vecs && vecs_out)
    for (uint64_t q = 0; q < n * num; ++q) vecs_out[q] = ritz[q];
  info->iterations = it;
  info->converged = conv ? 1 : 0;
  info->count = ev.size();
  info->num = num;
  return ok(err);
}

}  // namespace

extern "C" {

int or_power_iteration_f64(const uint64_t* indptr, const uint64_t* indices, const double* data, uint64_t n,
                           uint64_t max_iter, double tol, int normalize, const double* x0, uint64_t x0_len,
                           double* lambda, double* vec, double* resid, or_eig_info* info, or_err* err) {
  return power_iteration<double>({indptr, indices, n}, data, max_iter, tol, normalize, x0, x0_len, lambda, vec, resid,
                                 info, err);
}
int or_power_iteration_f32(const uint64_t* indptr, const uint64_t* indices, const float* data, uint64_t n,
                           uint64_t max_iter, double tol, int normalize, const float* x0, uint64_t x0_len,
                           float* lambda, float* vec, float* resid, or_eig_info* info, or_err* err) {
  return power_iteration<float>({indptr, indices, n}, data, max_iter, tol, normalize, x0, x0_len, lambda, vec, resid,
                                info, err);
}
int or_lanczos_f64(const uint64_t* indptr, const uint64_t* indices, const double* data, uint64_t n,
                   uint64_t max_iter, uint64_t max_subspace, double tol, uint64_t num_eigenvalues, int compute_vecs,
                   const double* v0, uint64_t v0_len, double* vals, double* vecs, double* resids, or_eig_info* info,
                   or_err* err) {
  return lanczos<double>({indptr, indices, n}, data, max_iter, max_subspace, tol, num_eigenvalues, compute_vecs, v0,
                         v0_len, vals, vecs, resids, info, err);
}
int or_lanczos_f32(const uint64_t* indptr, const uint64_t* indices, const float* data, uint64_t n, uint64_t max_iter,
                   uint64_t max_subspace, double tol, uint64_t num_eigenvalues, int compute_vecs, const float* v0,
                   uint64_t v0_len, float* vals, float* vecs, float* resids, or_eig_info* info, or_err* err) {
  return lanczos<float>({indptr, indices, n}, data, max_iter, max_subspace, tol, num_eigenvalues, compute_vecs, v0,
                        v0_len, vals, vecs, resids, info, err);
}
int or_tridiag_eig_f64(const double* alpha, const double* beta, uint64_t m, uint64_t beta_len, uint64_t num,
                       double* vals, double* vecs, uint64_t* count, or_err* err) {
  std::vector<double> a(alpha, alpha + m), b(beta, beta + beta_len), ev;
  std::vector<std::vector<double>> evec;
  const int rc = tridiag_eig<double>(a, b, num, ev, evec, err);
  if (rc) return rc;
  *count = ev.size();
  for (size_t k = 0; k < ev.size(); ++k) vals[k] = ev[k];
  for (size_t k = 0; k < evec.size(); ++k)
    for (size_t i = 0; i < evec[k].size(); ++i) vecs[k * m + i] = evec[k][i];
  return 0;
}
uint64_t or_solve_cubic_f64(double p, double q, double r, double* roots) {
  const std::vector<double> v = solve_cubic<double>(p, q, r);
  for (size_t k = 0; k < v.size(); ++k) roots[k] = v[k];
  return v.size();
}

}  // extern "C"
