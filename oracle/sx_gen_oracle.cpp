// CPU restatement of the library's seeded workload generators (test
// infrastructure, like the rest of oracle/).
//
// The reference crate has no PDE generators, so every large input of the
// benchmarks and of the config-size parity tests is produced by the
// library's own generator (scirs_gb300/csrc/sx_gen.cpp).  The reference arm
// of the benchmark and the CPU baselines must not load the device library,
// so this file restates the same generators, serially and independently of
// the device build: same random streams, same arithmetic in the same order
// (compiled with -ffp-contract=off like the library), so both give the same
// arrays bit for bit.  tests/test_oracle_gen.py checks that on the CPU.
//
// Random streams: splitmix64 (Steele, Lea and Flood, 2014).  A stream is
// seeded from (seed, stream index, tag); uniforms take the top 53 bits;
// normals use one Box-Muller draw (cosine branch) per value.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct Stream {
  uint64_t state;
  uint64_t next() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double gauss() {
    double a = unit();
    const double c = unit();
    a = a < 1e-300 ? 1e-300 : a;
    return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * c);
  }
};

Stream open_stream(uint64_t seed, uint64_t index, uint64_t tag) {
  Stream m{seed ^ (tag * 0xD1B54A32D192ED03ull)};
  m.state ^= index * 0x9E3779B97F4A7C15ull;
  m.next();
  return Stream{m.next()};
}

// normals in blocks of 4096 values, one stream per block
void block_normals(uint64_t seed, uint64_t tag, int64_t n, std::vector<double>& out, double scale,
                   bool exponentiate) {
  out.resize(n);
  for (int64_t b0 = 0; b0 < n; b0 += 4096) {
    Stream s = open_stream(seed, (uint64_t)(b0 / 4096), tag);
    const int64_t e = std::min<int64_t>(n, b0 + 4096);
    for (int64_t i = b0; i < e; ++i) {
      const double g = s.gauss();
      out[i] = exponentiate ? std::exp(scale * g) : g;
    }
  }
}

double harmonic(double a, double b) { return 2.0 * a * b / (a + b); }

// A row's (column, value) pairs, appended in ascending column order.
struct Rows {
  std::vector<int64_t> ptr{0};
  std::vector<int32_t> col;
  std::vector<double> val;
  void put(int64_t c, double v) { col.push_back((int32_t)c); val.push_back(v); }
  void end_row() { ptr.push_back((int64_t)col.size()); }
};

void gen_poisson2d(int64_t nx, int64_t ny, Rows& R) {
  for (int64_t y = 0; y < ny; ++y)
    for (int64_t x = 0; x < nx; ++x) {
      const int64_t i = y * nx + x;
      if (y > 0) R.put(i - nx, -1.0);
      if (x > 0) R.put(i - 1, -1.0);
      R.put(i, 4.0);
      if (x + 1 < nx) R.put(i + 1, -1.0);
      if (y + 1 < ny) R.put(i + nx, -1.0);
      R.end_row();
    }
}

void gen_laplace3d(int64_t nx, int64_t ny, int64_t nz, Rows& R) {
  const int64_t pl = nx * ny;
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x) {
        const int64_t i = z * pl + y * nx + x;
        if (z > 0) R.put(i - pl, -1.0);
        if (y > 0) R.put(i - nx, -1.0);
        if (x > 0) R.put(i - 1, -1.0);
        R.put(i, 6.0);
        if (x + 1 < nx) R.put(i + 1, -1.0);
        if (y + 1 < ny) R.put(i + nx, -1.0);
        if (z + 1 < nz) R.put(i + pl, -1.0);
        R.end_row();
      }
}

// Cell-centred diffusion with coefficient c = exp(sigma N(0,1)) per cell,
// harmonic means on interior faces and the cell's own c on boundary faces.
void gen_varcoef(int64_t nx, int64_t ny, int64_t nz, bool three_d, uint64_t seed, double sigma, Rows& R) {
  const int64_t n = nx * ny * nz, pl = nx * ny;
  std::vector<double> c;
  block_normals(seed, 0xC0EF, n, c, sigma, true);
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x) {
        const int64_t i = z * pl + y * nx + x;
        const double ci = c[i];
        const double f_zm = three_d ? (z > 0 ? harmonic(ci, c[i - pl]) : ci) : 0.0;
        const double f_ym = y > 0 ? harmonic(ci, c[i - nx]) : ci;
        const double f_xm = x > 0 ? harmonic(ci, c[i - 1]) : ci;
        const double f_xp = x + 1 < nx ? harmonic(ci, c[i + 1]) : ci;
        const double f_yp = y + 1 < ny ? harmonic(ci, c[i + nx]) : ci;
        const double f_zp = three_d ? (z + 1 < nz ? harmonic(ci, c[i + pl]) : ci) : 0.0;
        const double centre = f_xm + f_xp + f_ym + f_yp + (three_d ? f_zm + f_zp : 0.0);
        if (three_d && z > 0) R.put(i - pl, -f_zm);
        if (y > 0) R.put(i - nx, -f_ym);
        if (x > 0) R.put(i - 1, -f_xm);
        R.put(i, centre);
        if (x + 1 < nx) R.put(i + 1, -f_xp);
        if (y + 1 < ny) R.put(i + nx, -f_yp);
        if (three_d && z + 1 < nz) R.put(i + pl, -f_zp);
        R.end_row();
      }
}

// Q1 (bilinear) elements for -div(K grad u), K = R(theta) diag(1, 1/eps)
// R(theta)^T, on a uniform grid; the 9-point stencil is the sum, over the
// four cells around a node, of the cell's element-matrix row of that node.
void gen_aniso_q1(int64_t nx, int64_t ny, double eps, double theta, Rows& R) {
  const double cs = std::cos(theta), sn = std::sin(theta);
  const double l1 = 1.0, l2 = 1.0 / eps;
  const double kxx = cs * cs * l1 + sn * sn * l2;
  const double kyy = sn * sn * l1 + cs * cs * l2;
  const double kxy = cs * sn * (l1 - l2);
  // element matrix x 12, local corner l = a + 2 b
  const double dA = 4 * kxx + 6 * kxy + 4 * kyy, dB = 4 * kxx - 6 * kxy + 4 * kyy;
  const double hx = -4 * kxx + 2 * kyy, hy = 2 * kxx - 4 * kyy;
  const double g03 = -2 * kxx - 6 * kxy - 2 * kyy, g12 = -2 * kxx + 6 * kxy - 2 * kyy;
  const double E[4][4] = {{dA, hx, hy, g03}, {hx, dB, g12, hy}, {hy, g12, dB, hx}, {g03, hy, hx, dA}};
  double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int cb = 0; cb < 2; ++cb)
    for (int ca = 0; ca < 2; ++ca)
      for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) st[b - cb + 1][a - ca + 1] += E[ca + 2 * cb][a + 2 * b] / 12.0;
  for (int64_t y = 0; y < ny; ++y)
    for (int64_t x = 0; x < nx; ++x) {
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int64_t X = x + dx, Y = y + dy;
          if (X >= 0 && X < nx && Y >= 0 && Y < ny) R.put(Y * nx + X, st[dy + 1][dx + 1]);
        }
      R.end_row();
    }
}

// Rows with power-law lengths P(k) ~ k^-alpha on [1, kmax] (alpha found by
// bisection so that the mean length is `mean`), distinct uniform columns
// (drawn, sorted, deduplicated and topped up), values U(-1, 1).
int gen_powerlaw(int64_t n, uint64_t seed, double mean, int64_t kmax, Rows& R) {
  if (kmax > n) kmax = n;
  if (mean >= (double)kmax) return 2;
  auto mean_len = [&](double a) {
    double z = 0, m = 0;
    for (int64_t k = 1; k <= kmax; ++k) {
      const double w = std::pow((double)k, -a);
      z += w;
      m += w * k;
    }
    return m / z;
  };
  double lo = 0.0, hi = 8.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mean_len(mid) > mean) lo = mid;
    else hi = mid;
  }
  const double alpha = 0.5 * (lo + hi);
  std::vector<double> cdf(kmax);
  double z = 0;
  for (int64_t k = 1; k <= kmax; ++k) {
    z += std::pow((double)k, -alpha);
    cdf[k - 1] = z;
  }
  for (int64_t k = 0; k < kmax; ++k) cdf[k] /= z;
  cdf[kmax - 1] = 1.0;
  std::vector<int32_t> cols;
  for (int64_t i = 0; i < n; ++i) {
    Stream ls = open_stream(seed, (uint64_t)i, 0x1E4);
    const double u = ls.unit();
    int64_t len = (int64_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
    if (len > kmax) len = kmax;
    Stream cs = open_stream(seed, (uint64_t)i, 0xC015);
    cols.clear();
    while ((int64_t)cols.size() < len) {
      while ((int64_t)cols.size() < len) cols.push_back((int32_t)(cs.next() % (uint64_t)n));
      std::sort(cols.begin(), cols.end());
      cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    }
    for (int64_t j = 0; j < len; ++j) R.put(cols[j], 2.0 * cs.unit() - 1.0);
    R.end_row();
  }
  return 0;
}

}  // namespace

extern "C" {

// kind: 0 poisson2d, 1 laplace3d, 2 varcoef3d, 3 varcoef2d, 4 aniso_q1,
// 5 powerlaw (the library's sx_gen_kind numbering).  Fills *n and *nnz; with
// non-null arrays (n + 1, nnz, nnz entries) also the CSR.  0 on success.
int or_gen_matrix(int kind, int64_t nx, int64_t ny, int64_t nz, uint64_t seed, double p0, double p1,
                  int64_t* n_out, int64_t* nnz_out, int64_t* indptr, int32_t* indices, double* vals) {
  Rows R;
  int rc = 0;
  switch (kind) {
    case 0:
      if (nx <= 0 || ny <= 0) return 2;
      gen_poisson2d(nx, ny, R);
      break;
    case 1:
      if (nx <= 0 || ny <= 0 || nz <= 0) return 2;
      gen_laplace3d(nx, ny, nz, R);
      break;
    case 2:
    case 3: {
      const bool three = kind == 2;
      const int64_t NZ = three ? nz : 1;
      if (nx <= 0 || ny <= 0 || NZ <= 0) return 2;
      gen_varcoef(nx, ny, NZ, three, seed, p0 > 0 ? p0 : 1.0, R);
      break;
    }
    case 4:
      if (nx <= 0 || ny <= 0) return 2;
      gen_aniso_q1(nx, ny, p0 > 0 ? p0 : 1.0, p1, R);
      break;
    case 5:
      if (nx <= 0) return 2;
      rc = gen_powerlaw(nx, seed, p0 > 0 ? p0 : 16.0, p1 > 0 ? (int64_t)p1 : 4096, R);
      if (rc) return rc;
      break;
    default:
      return 4;
  }
  const int64_t n = (int64_t)R.ptr.size() - 1;
  *n_out = n;
  *nnz_out = (int64_t)R.col.size();
  if (indptr) {
    std::copy(R.ptr.begin(), R.ptr.end(), indptr);
    std::copy(R.col.begin(), R.col.end(), indices);
    std::copy(R.val.begin(), R.val.end(), vals);
  }
  return 0;
}

// Side of each system of the batched workload: uniform in [side_min, side_max].
void or_gen_batch_sides(uint64_t nsys, int64_t side_min, int64_t side_max, uint64_t seed, int64_t* sides) {
  for (uint64_t s = 0; s < nsys; ++s) {
    Stream r = open_stream(seed, s, 0x5AD);
    int64_t side = side_min + (int64_t)(r.unit() * (double)(side_max - side_min + 1));
    sides[s] = side > side_max ? side_max : side;
  }
}

// Seed of system s's coefficient field in the batched workload.
uint64_t or_gen_batch_system_seed(uint64_t seed, uint64_t s) { return seed * 0x9E3779B97F4A7C15ull + s + 1; }

// b_i ~ N(0, 1): blocks of 4096 values share one stream.
void or_gen_rhs_normal(uint64_t seed, int64_t n, double* b) {
  std::vector<double> v;
  block_normals(seed, 0xB0B, n, v, 1.0, false);
  std::copy(v.begin(), v.end(), b);
}

}  // extern "C"
