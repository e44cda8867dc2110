// Seeded synthetic workload generators for the sparse iterative-solve path.
//
// The reference crate ships no PDE generators (its tests build 2x2..10x10
// matrices inline, scirs2-sparse/tests/*.rs), so every large input of this
// library comes from here.  All generators are host code, deterministic for a
// given seed and independent of the thread count: each row draws from its own
// counter-derived splitmix64 stream.
//
// Matrices come out as CSR with int64 row pointers, int32 column indices
// (sorted within each row, no duplicates) and FP64 values.  Rows follow the
// natural (x fastest) ordering; Dirichlet boundary nodes are eliminated.

#include "scirs_sparse_gen.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// splitmix64 (Steele, Lea, Flood 2014): one 64-bit state, one output per step.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // standard normal by the Box-Muller transform (one value per call)
  double normal() {
    double u1 = uniform();
    double u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

uint64_t stream_seed(uint64_t seed, uint64_t stream, uint64_t tag) {
  SplitMix64 m(seed ^ (tag * 0xD1B54A32D192ED03ull));
  m.s ^= stream * 0x9E3779B97F4A7C15ull;
  m.next();
  return m.next();
}

template <class Fn>
void parallel_rows(int64_t n, Fn fn) {
  unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = hw ? (int64_t)hw : 4;
  if (nt > 64) nt = 64;
  if (n < 65536) nt = 1;
  std::vector<std::thread> th;
  int64_t chunk = (n + nt - 1) / nt;
  for (int64_t t = 0; t < nt; ++t) {
    int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([=]() { fn(lo, hi); });
  }
  for (auto& t : th) t.join();
}

// ---------------------------------------------------------------- stencils
// Generic constant or variable stencil assembly: for each row, the callback
// writes (col, value) pairs in ascending column order.

struct Dims { int64_t nx, ny, nz; };

int64_t stencil5_nnz(int64_t nx, int64_t ny) { return 5 * nx * ny - 2 * nx - 2 * ny; }
int64_t stencil7_nnz(int64_t nx, int64_t ny, int64_t nz) {
  return 7 * nx * ny * nz - 2 * (nx * ny + ny * nz + nx * nz);
}
int64_t stencil9_nnz(int64_t nx, int64_t ny) {
  // 9 per row minus the missing neighbours of boundary nodes
  if (nx <= 0 || ny <= 0) return 0;
  int64_t n = nx * ny;
  // each boundary side removes 3 per node, corners double counted (+1 each)
  int64_t removed = 3 * nx * 2 + 3 * ny * 2 - 4;
  if (nx == 1 || ny == 1) {
    // degenerate strips: count directly
    int64_t c = 0;
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            int64_t X = x + dx, Y = y + dy;
            if (X >= 0 && X < nx && Y >= 0 && Y < ny) ++c;
          }
    return c;
  }
  return 9 * n - removed;
}

// harmonic mean of two positive face coefficients
inline double harm(double a, double b) { return 2.0 * a * b / (a + b); }

}  // namespace

extern "C" {

void sx_gen_rhs_normal(uint64_t seed, int64_t n, double* b) {
  parallel_rows(n, [&](int64_t lo, int64_t hi) {
    // blocks of 4096 values share one stream so the result is thread-count independent
    for (int64_t blk = lo / 4096; blk * 4096 < hi; ++blk) {
      SplitMix64 r(stream_seed(seed, (uint64_t)blk, 0xB0B));
      int64_t s = blk * 4096, e = std::min(hi, s + 4096);
      for (int64_t i = blk * 4096; i < e; ++i) {
        double v = r.normal();
        if (i >= lo) b[i] = v;
      }
    }
  });
}

int sx_gen_matrix(const sx_gen_spec* spec, int64_t* n_out, int64_t* nnz_out, int64_t* indptr,
                  int32_t* indices, double* vals) {
  if (!spec || !n_out || !nnz_out) return 1;
  const int64_t nx = spec->nx, ny = spec->ny, nz = spec->nz;
  switch (spec->kind) {
    case SX_GEN_POISSON2D: {
      if (nx <= 0 || ny <= 0) return 2;
      int64_t n = nx * ny, nnz = stencil5_nnz(nx, ny);
      *n_out = n; *nnz_out = nnz;
      if (!indptr) return 0;
      int64_t k = 0;
      for (int64_t i = 0; i < n; ++i) {
        int64_t x = i % nx, y = i / nx;
        indptr[i] = k;
        if (y > 0) { indices[k] = (int32_t)(i - nx); vals[k++] = -1.0; }
        if (x > 0) { indices[k] = (int32_t)(i - 1); vals[k++] = -1.0; }
        indices[k] = (int32_t)i; vals[k++] = 4.0;
        if (x < nx - 1) { indices[k] = (int32_t)(i + 1); vals[k++] = -1.0; }
        if (y < ny - 1) { indices[k] = (int32_t)(i + nx); vals[k++] = -1.0; }
      }
      indptr[n] = k;
      return k == nnz ? 0 : 3;
    }
    case SX_GEN_LAPLACE3D: {
      if (nx <= 0 || ny <= 0 || nz <= 0) return 2;
      int64_t n = nx * ny * nz, nnz = stencil7_nnz(nx, ny, nz);
      *n_out = n; *nnz_out = nnz;
      if (!indptr) return 0;
      const int64_t sxy = nx * ny;
      // per-row counts are known in closed form; compute prefix on one thread
      int64_t k = 0;
      for (int64_t i = 0; i < n; ++i) {
        int64_t x = i % nx, y = (i / nx) % ny, z = i / sxy;
        indptr[i] = k;
        k += 1 + (z > 0) + (y > 0) + (x > 0) + (x < nx - 1) + (y < ny - 1) + (z < nz - 1);
      }
      indptr[n] = k;
      parallel_rows(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
          int64_t x = i % nx, y = (i / nx) % ny, z = i / sxy;
          int64_t p = indptr[i];
          if (z > 0) { indices[p] = (int32_t)(i - sxy); vals[p++] = -1.0; }
          if (y > 0) { indices[p] = (int32_t)(i - nx); vals[p++] = -1.0; }
          if (x > 0) { indices[p] = (int32_t)(i - 1); vals[p++] = -1.0; }
          indices[p] = (int32_t)i; vals[p++] = 6.0;
          if (x < nx - 1) { indices[p] = (int32_t)(i + 1); vals[p++] = -1.0; }
          if (y < ny - 1) { indices[p] = (int32_t)(i + nx); vals[p++] = -1.0; }
          if (z < nz - 1) { indices[p] = (int32_t)(i + sxy); vals[p++] = -1.0; }
        }
      });
      return k == nnz ? 0 : 3;
    }
    case SX_GEN_VARCOEF3D:
    case SX_GEN_VARCOEF2D: {
      const bool is3 = spec->kind == SX_GEN_VARCOEF3D;
      const int64_t NZ = is3 ? nz : 1;
      if (nx <= 0 || ny <= 0 || NZ <= 0) return 2;
      int64_t n = nx * ny * NZ;
      int64_t nnz = is3 ? stencil7_nnz(nx, ny, NZ) : stencil5_nnz(nx, ny);
      *n_out = n; *nnz_out = nnz;
      if (!indptr) return 0;
      const double sigma = spec->param0 > 0 ? spec->param0 : 1.0;
      // cell coefficients c = exp(sigma * N(0,1)), one stream per block of cells
      std::vector<double> c(n);
      parallel_rows(n, [&](int64_t lo, int64_t hi) {
        for (int64_t blk = lo / 4096; blk * 4096 < hi; ++blk) {
          SplitMix64 r(stream_seed(spec->seed, (uint64_t)blk, 0xC0EF));
          int64_t e = std::min(hi, blk * 4096 + 4096);
          for (int64_t i = blk * 4096; i < e; ++i) {
            double v = std::exp(sigma * r.normal());
            if (i >= lo) c[i] = v;
          }
        }
      });
      const int64_t sxy = nx * ny;
      int64_t k = 0;
      for (int64_t i = 0; i < n; ++i) {
        int64_t x = i % nx, y = (i / nx) % ny, z = i / sxy;
        indptr[i] = k;
        k += 1 + (x > 0) + (x < nx - 1) + (y > 0) + (y < ny - 1);
        if (is3) k += (z > 0) + (z < NZ - 1);
      }
      indptr[n] = k;
      parallel_rows(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
          int64_t x = i % nx, y = (i / nx) % ny, z = i / sxy;
          int64_t p = indptr[i];
          const double ci = c[i];
          double diag = 0.0;
          // faces in ascending column order; boundary faces use the cell's own c
          double fzm = 0, fym = 0, fxm = 0, fxp = 0, fyp = 0, fzp = 0;
          if (is3) fzm = z > 0 ? harm(ci, c[i - sxy]) : ci;
          fym = y > 0 ? harm(ci, c[i - nx]) : ci;
          fxm = x > 0 ? harm(ci, c[i - 1]) : ci;
          fxp = x < nx - 1 ? harm(ci, c[i + 1]) : ci;
          fyp = y < ny - 1 ? harm(ci, c[i + nx]) : ci;
          if (is3) fzp = z < NZ - 1 ? harm(ci, c[i + sxy]) : ci;
          diag = fxm + fxp + fym + fyp + (is3 ? fzm + fzp : 0.0);
          if (is3 && z > 0) { indices[p] = (int32_t)(i - sxy); vals[p++] = -fzm; }
          if (y > 0) { indices[p] = (int32_t)(i - nx); vals[p++] = -fym; }
          if (x > 0) { indices[p] = (int32_t)(i - 1); vals[p++] = -fxm; }
          indices[p] = (int32_t)i; vals[p++] = diag;
          if (x < nx - 1) { indices[p] = (int32_t)(i + 1); vals[p++] = -fxp; }
          if (y < ny - 1) { indices[p] = (int32_t)(i + nx); vals[p++] = -fyp; }
          if (is3 && z < NZ - 1) { indices[p] = (int32_t)(i + sxy); vals[p++] = -fzp; }
        }
      });
      return k == nnz ? 0 : 3;
    }
    case SX_GEN_ANISO_Q1: {
      // Bilinear (Q1) finite elements for -div(K grad u) on a uniform grid with
      // K = R(theta) diag(1, 1/eps) R(theta)^T.  The element matrix of a
      // square cell (independent of h in 2D), local node l = a + 2b at
      // corner (a, b), times 12:
      //   d0 = 4kxx+6kxy+4kyy (corners 0,3)  d1 = 4kxx-6kxy+4kyy (corners 1,2)
      //   e01 = e23 = -4kxx+2kyy   e02 = e13 = 2kxx-4kyy
      //   e03 = -2kxx-6kxy-2kyy   e12 = -2kxx+6kxy-2kyy
      if (nx <= 0 || ny <= 0) return 2;
      const double eps = spec->param0 > 0 ? spec->param0 : 1.0;
      const double th = spec->param1;
      const double cs = std::cos(th), sn = std::sin(th);
      const double l1 = 1.0, l2 = 1.0 / eps;
      const double kxx = cs * cs * l1 + sn * sn * l2;
      const double kyy = sn * sn * l1 + cs * cs * l2;
      const double kxy = cs * sn * (l1 - l2);
      double E[4][4];
      const double d0 = 4 * kxx + 6 * kxy + 4 * kyy, d1 = 4 * kxx - 6 * kxy + 4 * kyy;
      const double e01 = -4 * kxx + 2 * kyy, e02 = 2 * kxx - 4 * kyy;
      const double e03 = -2 * kxx - 6 * kxy - 2 * kyy, e12 = -2 * kxx + 6 * kxy - 2 * kyy;
      E[0][0] = d0; E[3][3] = d0; E[1][1] = d1; E[2][2] = d1;
      E[0][1] = E[1][0] = e01; E[2][3] = E[3][2] = e01;
      E[0][2] = E[2][0] = e02; E[1][3] = E[3][1] = e02;
      E[0][3] = E[3][0] = e03; E[1][2] = E[2][1] = e12;
      // 9-point stencil S[dy+1][dx+1]: sum over the 4 cells around a node
      double S[3][3] = {{0}};
      for (int cb = 0; cb < 2; ++cb)
        for (int ca = 0; ca < 2; ++ca) {
          // cell whose corner (ca, cb) is the centre node
          int lc = ca + 2 * cb;
          for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
              int l = a + 2 * b;
              S[b - cb + 1][a - ca + 1] += E[lc][l] / 12.0;
            }
        }
      int64_t n = nx * ny, nnz = stencil9_nnz(nx, ny);
      *n_out = n; *nnz_out = nnz;
      if (!indptr) return 0;
      int64_t k = 0;
      for (int64_t i = 0; i < n; ++i) {
        int64_t x = i % nx, y = i / nx;
        indptr[i] = k;
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            int64_t X = x + dx, Y = y + dy;
            if (X >= 0 && X < nx && Y >= 0 && Y < ny) ++k;
          }
      }
      indptr[n] = k;
      parallel_rows(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
          int64_t x = i % nx, y = i / nx;
          int64_t p = indptr[i];
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              int64_t X = x + dx, Y = y + dy;
              if (X >= 0 && X < nx && Y >= 0 && Y < ny) {
                indices[p] = (int32_t)(Y * nx + X);
                vals[p++] = S[dy + 1][dx + 1];
              }
            }
        }
      });
      return k == nnz ? 0 : 3;
    }
    case SX_GEN_POWERLAW: {
      // Row lengths from a discrete power law P(k) ~ k^-alpha on [1, kmax],
      // alpha fitted by bisection so that E[k] = mean.  Columns uniform
      // without replacement within a row, sorted; values U(-1, 1).
      const int64_t n = nx;
      if (n <= 0) return 2;
      const double mean = spec->param0 > 0 ? spec->param0 : 16.0;
      int64_t kmax = spec->param1 > 0 ? (int64_t)spec->param1 : 4096;
      if (kmax > n) kmax = n;
      if (mean >= (double)kmax) return 2;
      std::vector<double> cdf(kmax);
      auto mean_of = [&](double a) {
        double z = 0, m = 0;
        for (int64_t k = 1; k <= kmax; ++k) { double w = std::pow((double)k, -a); z += w; m += w * k; }
        return m / z;
      };
      double lo = 0.0, hi = 8.0;
      for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mean_of(mid) > mean) lo = mid; else hi = mid;
      }
      const double alpha = 0.5 * (lo + hi);
      {
        double z = 0;
        for (int64_t k = 1; k <= kmax; ++k) { z += std::pow((double)k, -alpha); cdf[k - 1] = z; }
        for (int64_t k = 0; k < kmax; ++k) cdf[k] /= z;
        cdf[kmax - 1] = 1.0;
      }
      std::vector<int32_t> len(n);
      parallel_rows(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i) {
          SplitMix64 r(stream_seed(spec->seed, (uint64_t)i, 0x1E4));
          double u = r.uniform();
          len[i] = (int32_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
          if (len[i] > kmax) len[i] = (int32_t)kmax;
        }
      });
      int64_t k = 0;
      if (indptr) {
        for (int64_t i = 0; i < n; ++i) { indptr[i] = k; k += len[i]; }
        indptr[n] = k;
      } else {
        for (int64_t i = 0; i < n; ++i) k += len[i];
      }
      *n_out = n; *nnz_out = k;
      if (!indptr) return 0;
      parallel_rows(n, [&](int64_t a, int64_t b) {
        std::vector<int32_t> cols;
        for (int64_t i = a; i < b; ++i) {
          SplitMix64 r(stream_seed(spec->seed, (uint64_t)i, 0xC015));
          int32_t L = len[i];
          cols.clear();
          // draw, sort, dedupe, top up until L distinct columns
          while ((int32_t)cols.size() < L) {
            while ((int32_t)cols.size() < L) cols.push_back((int32_t)(r.next() % (uint64_t)n));
            std::sort(cols.begin(), cols.end());
            cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
          }
          int64_t p = indptr[i];
          for (int32_t j = 0; j < L; ++j) {
            indices[p + j] = cols[j];
            vals[p + j] = 2.0 * r.uniform() - 1.0;
          }
        }
      });
      return 0;
    }
    default:
      return 4;
  }
}

int sx_gen_batch_varcoef2d(uint64_t nsys, int64_t side_min, int64_t side_max, uint64_t seed,
                           double sigma, int64_t* sys_ptr, int64_t* n_out, int64_t* nnz_out,
                           int64_t* indptr, int32_t* indices, double* vals) {
  if (!sys_ptr || !n_out || !nnz_out || side_min < 1 || side_max < side_min) return 2;
  std::vector<int64_t> side(nsys), nnz_ptr(nsys + 1, 0);
  sys_ptr[0] = 0;
  for (uint64_t s = 0; s < nsys; ++s) {
    SplitMix64 r(stream_seed(seed, s, 0x5AD));
    side[s] = side_min + (int64_t)(r.uniform() * (double)(side_max - side_min + 1));
    if (side[s] > side_max) side[s] = side_max;
    sys_ptr[s + 1] = sys_ptr[s] + side[s] * side[s];
    nnz_ptr[s + 1] = nnz_ptr[s] + stencil5_nnz(side[s], side[s]);
  }
  *n_out = sys_ptr[nsys];
  *nnz_out = nnz_ptr[nsys];
  if (!indptr) return 0;
  // systems in parallel; each writes its own slice with global numbering
  unsigned hw = std::thread::hardware_concurrency();
  int nt = hw ? (int)std::min<unsigned>(hw, 64) : 4;
  std::vector<std::thread> th;
  std::vector<int> rc(nt, 0);
  for (int t = 0; t < nt; ++t) {
    th.emplace_back([&, t]() {
      for (uint64_t s = t; s < nsys; s += nt) {
        sx_gen_spec sp{SX_GEN_VARCOEF2D, side[s], side[s], 1, seed * 0x9E3779B97F4A7C15ull + s + 1, sigma, 0.0};
        int64_t n = 0, nnz = 0;
        const int64_t r0 = sys_ptr[s], k0 = nnz_ptr[s];
        std::vector<int64_t> ip(side[s] * side[s] + 1);
        int e = sx_gen_matrix(&sp, &n, &nnz, ip.data(), indices + k0, vals + k0);
        if (e) { rc[t] = e; return; }
        for (int64_t i = 0; i < n; ++i) indptr[r0 + i] = ip[i] + k0;
        for (int64_t k = 0; k < nnz; ++k) indices[k0 + k] += (int32_t)r0;
      }
    });
  }
  for (auto& x : th) x.join();
  indptr[*n_out] = *nnz_out;
  for (int e : rc)
    if (e) return e;
  return 0;
}

}  // extern "C"
