// Learned factorised sparse approximate inverse (no reference counterpart;
// its nearest relative in the reference is SpaiPreconditioner,
// scirs2-sparse/src/linalg/spai.rs:15-192, a different method).
//
// A message-passing network over the graph of A (nodes = rows, edges =
// nonzeros) predicts a lower-triangular G on the pattern of lower(A) with a
// softplus diagonal, so M^-1 = G G^T is SPD; it is applied as two SpMVs.
//
// The network works on the Jacobi-scaled matrix A^ = D^-1/2 A D^-1/2 (unit
// diagonal), so G^ = I is exactly Jacobi; G = D^-1/2 G^.
//   node features  x_i = [1, sum_j |a^_ij|, sum_j a^_ij, max_j |a^_ij|]
//   3 layers       h' = ReLU(W_s h_i + sum_j a^_ij W_n h_j + b), hidden 64
//   off-diagonal   g^_ij = q . ReLU(P1 h_i + P2 h_j + p3 a^_ij + p0), j < i
//   diagonal       g^_ii = softplus(w_d . h_i + b_d)
// Dense layers: BF16 weights and BF16 inputs on the tensor cores
// (mma.sync m16n8k16), FP32 accumulation.
// Training loss: ||(G^T A^ G - I) Z||_F^2 / (k n) over k Gaussian probes;
// gradient on the pattern: 2/(k n) (W_i . R_j + Q_i . Z_j) with
// W = A^ G Z, R = G^T W - Z, Q = A^ G R; backward through the heads and the
// layers is hand-written below, all reductions deterministic.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "sx_launch.cuh"

namespace sx {
namespace gnn {

constexpr int kF0 = 4;    // node features
constexpr int kK0 = 16;   // padded GEMM input width of layer 0
constexpr int kH = 64;    // hidden width
constexpr int kL = 3;     // message-passing layers
constexpr int kC = 32;    // edge-head width
constexpr int kNH = 72;   // head GEMM rows: P1 (32), P2 (32), w_d (1), zero pad (7)
constexpr int kP = 4;     // probes per training step
constexpr int kGemmRows = 64;

typedef __nv_bfloat16 bf16;

// ----------------------------------------------------- parameter layout
struct Layout {
  int ws[kL], wn[kL], b[kL], kin[kL];
  int P1, P2, p3, p0, q, wd, bd, total;
};
Layout layout() {
  Layout L;
  int o = 0, kin = kF0;
  for (int l = 0; l < kL; ++l) {
    L.kin[l] = kin;
    L.ws[l] = o; o += kH * kin;
    L.wn[l] = o; o += kH * kin;
    L.b[l] = o; o += kH;
    kin = kH;
  }
  L.P1 = o; o += kC * kH;
  L.P2 = o; o += kC * kH;
  L.p3 = o; o += kC;
  L.p0 = o; o += kC;
  L.q = o; o += kC;
  L.wd = o; o += kH;
  L.bd = o; o += 1;
  L.total = o;
  return L;
}

// ------------------------------------------------------- per-matrix data
struct Graph {
  uint64_t key = 0;
  int64_t n = 0, noff = 0, ng = 0;
  float* dis = nullptr;                       // D^-1/2
  int32_t *op = nullptr, *oi = nullptr;       // off-diagonal A^ (CSR)
  float* ov = nullptr;
  bf16* x0 = nullptr;                         // n x kK0 node features
  int32_t *gp = nullptr, *gi = nullptr;       // G pattern: strict lower, then diagonal
  float* ga = nullptr;                        // a^ of each G entry (0 on the diagonal)
  int32_t *tp = nullptr, *ti = nullptr, *tperm = nullptr;  // G^T pattern -> G entry
};

void graph_free(Graph& g) {
  dev_free(g.dis); dev_free(g.op); dev_free(g.oi); dev_free(g.ov); dev_free(g.x0);
  dev_free(g.gp); dev_free(g.gi); dev_free(g.ga); dev_free(g.tp); dev_free(g.ti); dev_free(g.tperm);
  g = Graph{};
}

struct Acts {
  int64_t n = 0, ng = 0;
  bf16* h[kL + 1] = {nullptr};   // h[0] aliases the graph's x0
  float* pre[kL] = {nullptr};    // n x kH pre-activations
  float* S = nullptr;            // n x 2kH layer GEMM output / its gradient
  float* Y = nullptr;            // n x kNH head GEMM output
  float* dY = nullptr;           // n x kNH
  float* dH = nullptr;           // n x kH
  float* dH2 = nullptr;          // n x kH
  float* g = nullptr;            // ng edge values
  float* dg = nullptr;           // ng
  float* dz = nullptr;           // ng x kC
  float *Z = nullptr, *Yp = nullptr, *W = nullptr, *V = nullptr, *R = nullptr, *Pp = nullptr,
        *Q = nullptr;            // n x kP probe vectors
  float* part = nullptr;         // reduction partials
  size_t part_floats = 0;
  float* dw = nullptr;           // one weight gradient [<= 2kH x kH]
};

}  // namespace gnn
}  // namespace sx

struct sx_gnn_s {
  int device = 0;
  sx::gnn::Layout L;
  float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  sx::gnn::bf16* wc[sx::gnn::kL] = {nullptr};  // [2kH x kpad] per layer
  sx::gnn::bf16* wh = nullptr;                 // [kNH x kH]
  float* wcf[sx::gnn::kL] = {nullptr};         // BF16-rounded weights as FP32 (backward)
  float* whf = nullptr;
  int step = 0;
  std::vector<sx::gnn::Graph> graphs;
  sx::gnn::Acts acts;
  float* loss = nullptr;                       // device scalar
  unsigned int* counter = nullptr;
};

namespace sx {
namespace gnn {

// ================================================================ kernels
__device__ __forceinline__ float softplus(float t) { return t > 20.f ? t : log1pf(expf(t)); }
__device__ __forceinline__ float dsoftplus(float t) { return t > 20.f ? 1.f : 1.f / (1.f + expf(-t)); }

// --- preparation -------------------------------------------------------
template <typename T>
__global__ void k_dis(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                      const T* __restrict__ val, int64_t n, float* dis, int* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
      if (idx[k] == (int32_t)i) { d = (double)val[k]; break; }
    if (!(d > 0.0)) *bad = 1;
    dis[i] = (float)(1.0 / sqrt(d));
  }
}

__global__ void k_count_off_lower(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                  int64_t n, int32_t* off_cnt, int32_t* g_cnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t off = 0, low = 0;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      off += idx[k] != (int32_t)i;
      low += idx[k] < (int32_t)i;
    }
    off_cnt[i] = off;
    g_cnt[i] = low + 1;
  }
}

// position of column c in row r (columns strictly increasing), or -1
__device__ __forceinline__ int32_t row_find(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                            int32_t r, int32_t c) {
  int32_t lo = ptr[r], hi = ptr[r + 1];
  while (lo < hi) {
    const int32_t mid = lo + (hi - lo) / 2;
    if (idx[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return lo < ptr[r + 1] && idx[lo] == c ? lo : -1;
}

// Structurally symmetric A (every row's columns strictly increasing, and
// (j, i) stored for every stored (i, j)): the transpose of G's pattern (each
// row's strict-lower columns, then the diagonal) has in row j the diagonal
// and then row j's upper columns, in that order.  flag is set when A is not
// such a matrix; t_cnt[j] = row j's upper entries + 1.
__global__ void k_sym_pattern(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                              int32_t* t_cnt, int* flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t up = 0, prev = -1;
    bool bad = false;
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int32_t j = idx[k];
      if (j <= prev || j < 0 || j >= n) {
        bad = true;
        break;
      }
      prev = j;
      up += j > (int32_t)i;
      if (row_find(ptr, idx, j, (int32_t)i) < 0) bad = true;
    }
    t_cnt[i] = up + 1;
    if (bad) *flag = 1;
  }
}

// G^T's pattern and entry map (G^T entry -> G entry) of a structurally
// symmetric A: entry (j, j) is G's last entry of row j; entry (j, i), i > j,
// is G's entry of column j in row i, whose strict-lower columns are row i's
// first ones
__global__ void k_gt_from_sym(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                              const int32_t* __restrict__ gp, const int32_t* __restrict__ tp, int32_t* ti,
                              int32_t* tperm) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    int32_t t = tp[j];
    ti[t] = (int32_t)j;
    tperm[t] = gp[j + 1] - 1;
    ++t;
    for (int32_t k = ptr[j]; k < ptr[j + 1]; ++k) {
      const int32_t i = idx[k];
      if (i <= (int32_t)j) continue;
      ti[t] = i;
      tperm[t] = gp[i] + (row_find(ptr, idx, i, (int32_t)j) - ptr[i]);
      ++t;
    }
  }
}

template <typename T>
__global__ void k_fill_graph(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const T* __restrict__ val, int64_t n, const float* __restrict__ dis,
                             const int32_t* __restrict__ op, int32_t* oi, float* ov,
                             const int32_t* __restrict__ gp, int32_t* gi, float* ga, bf16* x0,
                             double* gidx) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t o = op[i], g = gp[i];
    float s_abs = 0.f, s_sgn = 0.f, s_max = 0.f;
    const float di = dis[i];
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int32_t j = idx[k];
      if (j == (int32_t)i) continue;
      const float a = ((float)val[k] * di) * dis[j];
      oi[o] = j;
      ov[o] = a;
      ++o;
      s_abs += fabsf(a);
      s_sgn += a;
      s_max = fmaxf(s_max, fabsf(a));
      if (j < (int32_t)i) {
        gi[g] = j;
        ga[g] = a;
        if (gidx) gidx[g] = (double)g;
        ++g;
      }
    }
    gi[g] = (int32_t)i;
    ga[g] = 0.f;
    if (gidx) gidx[g] = (double)g;
    bf16* xr = x0 + i * kK0;
    xr[0] = __float2bfloat16(1.f);
    xr[1] = __float2bfloat16(s_abs);
    xr[2] = __float2bfloat16(s_sgn);
    xr[3] = __float2bfloat16(s_max);
    for (int c = kF0; c < kK0; ++c) xr[c] = __float2bfloat16(0.f);
  }
}

__global__ void k_perm_from_double(const double* __restrict__ v, int64_t n, int32_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)v[i];
}

// --- tensor-core GEMM: C[M x N] = A[M x K] B[N x K]^T, BF16 in, FP32 out ---
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int K, int N>
__global__ void __launch_bounds__(128) k_gemm_bf16(const bf16* __restrict__ A, const bf16* __restrict__ B,
                                                   float* __restrict__ Cm, int64_t M) {
  __shared__ __align__(16) bf16 Bs[N * K];
  for (int i = threadIdx.x; i < N * K; i += blockDim.x) Bs[i] = B[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int64_t r0 = (int64_t)blockIdx.x * kGemmRows + warp * 16;
  const int64_t ra = r0 + g, rb = r0 + g + 8;
  float acc[N / 8][4];
#pragma unroll
  for (int j = 0; j < N / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < K; kk += 16) {
    uint32_t a[4];
    a[0] = ra < M ? *reinterpret_cast<const uint32_t*>(A + ra * K + kk + 2 * t) : 0u;
    a[1] = rb < M ? *reinterpret_cast<const uint32_t*>(A + rb * K + kk + 2 * t) : 0u;
    a[2] = ra < M ? *reinterpret_cast<const uint32_t*>(A + ra * K + kk + 8 + 2 * t) : 0u;
    a[3] = rb < M ? *reinterpret_cast<const uint32_t*>(A + rb * K + kk + 8 + 2 * t) : 0u;
#pragma unroll
    for (int j = 0; j < N / 8; ++j) {
      uint32_t b[2];
      b[0] = *reinterpret_cast<const uint32_t*>(Bs + (j * 8 + g) * K + kk + 2 * t);
      b[1] = *reinterpret_cast<const uint32_t*>(Bs + (j * 8 + g) * K + kk + 8 + 2 * t);
      mma_bf16(acc[j], a, b);
    }
  }
#pragma unroll
  for (int j = 0; j < N / 8; ++j) {
    if (ra < M) *reinterpret_cast<float2*>(Cm + ra * N + j * 8 + 2 * t) = make_float2(acc[j][0], acc[j][1]);
    if (rb < M) *reinterpret_cast<float2*>(Cm + rb * N + j * 8 + 2 * t) = make_float2(acc[j][2], acc[j][3]);
  }
}

// --- message passing: pre = S_self + sum_j a^_ij S_nb[j] + b; h = bf16(relu(pre))
// (pre is stored for the backward pass only: null when the network predicts)
__global__ void k_aggregate(const float* __restrict__ S, const int32_t* __restrict__ op,
                            const int32_t* __restrict__ oi, const float* __restrict__ ov,
                            const float* __restrict__ bias, int64_t n, float* pre, bf16* hout) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const float2 self = *reinterpret_cast<const float2*>(S + i * 2 * kH + 2 * lane);
    float ax = 0.f, ay = 0.f;
    for (int32_t e = op[i]; e < op[i + 1]; ++e) {
      const float a = ov[e];
      const float2 nb = *reinterpret_cast<const float2*>(S + (int64_t)oi[e] * 2 * kH + kH + 2 * lane);
      ax += a * nb.x;
      ay += a * nb.y;
    }
    const float px = self.x + ax + bias[2 * lane];
    const float py = self.y + ay + bias[2 * lane + 1];
    if (pre) *reinterpret_cast<float2*>(pre + i * kH + 2 * lane) = make_float2(px, py);
    hout[i * kH + 2 * lane] = __float2bfloat16(fmaxf(px, 0.f));
    hout[i * kH + 2 * lane + 1] = __float2bfloat16(fmaxf(py, 0.f));
  }
}

// --- heads: one warp per row, lane = head channel
__global__ void k_edge_head(const float* __restrict__ Y, const int32_t* __restrict__ gp,
                            const int32_t* __restrict__ gi, const float* __restrict__ ga,
                            const float* __restrict__ params, int p3o, int p0o, int qo, int bdo,
                            int64_t n, float* gval) {
  const int lane = threadIdx.x & 31;
  const float p3 = params[p3o + lane], p0 = params[p0o + lane], q = params[qo + lane];
  const float bd = params[bdo];
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const float y1 = Y[i * kNH + lane];
    for (int32_t e = gp[i]; e < gp[i + 1]; ++e) {
      const int32_t j = gi[e];
      if (j == (int32_t)i) {
        if (lane == 0) gval[e] = softplus(Y[i * kNH + 2 * kC] + bd);
      } else {
        const float z = fmaxf(y1 + Y[(int64_t)j * kNH + kC + lane] + ga[e] * p3 + p0, 0.f);
        const float s = warp_sum(z * q);
        if (lane == 0) gval[e] = s;
      }
    }
  }
}

// --- probe products (k = kP columns per row, row-major) -------------------
// Y = G Z
__global__ void k_spmm_g(const int32_t* __restrict__ gp, const int32_t* __restrict__ gi,
                         const float* __restrict__ g, const float* __restrict__ Z, int64_t n, float* Y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int32_t e = gp[i]; e < gp[i + 1]; ++e) {
      const float w = g[e];
      const float4 z = *reinterpret_cast<const float4*>(Z + (int64_t)gi[e] * kP);
      acc.x += w * z.x; acc.y += w * z.y; acc.z += w * z.z; acc.w += w * z.w;
    }
    *reinterpret_cast<float4*>(Y + i * kP) = acc;
  }
}
// W = A^ Y = Y + offdiag(A^) Y
__global__ void k_spmm_a(const int32_t* __restrict__ op, const int32_t* __restrict__ oi,
                         const float* __restrict__ ov, const float* __restrict__ Yi, int64_t n, float* W) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int32_t e = op[i]; e < op[i + 1]; ++e) {
      const float w = ov[e];
      const float4 z = *reinterpret_cast<const float4*>(Yi + (int64_t)oi[e] * kP);
      acc.x += w * z.x; acc.y += w * z.y; acc.z += w * z.z; acc.w += w * z.w;
    }
    const float4 s = *reinterpret_cast<const float4*>(Yi + i * kP);
    *reinterpret_cast<float4*>(W + i * kP) = make_float4(s.x + acc.x, s.y + acc.y, s.z + acc.z, s.w + acc.w);
  }
}
// V = G^T W through the transposed pattern
__global__ void k_spmm_gt(const int32_t* __restrict__ tp, const int32_t* __restrict__ ti,
                          const int32_t* __restrict__ tperm, const float* __restrict__ g,
                          const float* __restrict__ Wm, int64_t n, float* V) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int32_t t = tp[j]; t < tp[j + 1]; ++t) {
      const float w = g[tperm[t]];
      const float4 z = *reinterpret_cast<const float4*>(Wm + (int64_t)ti[t] * kP);
      acc.x += w * z.x; acc.y += w * z.y; acc.z += w * z.z; acc.w += w * z.w;
    }
    *reinterpret_cast<float4*>(V + j * kP) = acc;
  }
}
// R = V - Z, loss = sum R^2 / (k n)
__global__ void __launch_bounds__(kBlock) k_resid_loss(const float* __restrict__ V, const float* __restrict__ Z,
                                                       int64_t n, float* R, float* partials,
                                                       unsigned int* counter, float* loss) {
  Acc3<float> a{0.f, 0.f, 0.f};
  for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n * kP; i += (int64_t)gridDim.x * kBlock) {
    const float r = V[i] - Z[i];
    R[i] = r;
    a.a += r * r;
  }
  Acc3<float> tot;
  if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) *loss = tot.a / (float)(kP * n);
}
// dg_e = 2/(k n) sum_c (W_ic R_jc + Q_ic Z_jc)
__global__ void k_sddmm(const int32_t* __restrict__ gp, const int32_t* __restrict__ gi,
                        const float* __restrict__ Wm, const float* __restrict__ R,
                        const float* __restrict__ Q, const float* __restrict__ Z, int64_t n, float scale,
                        float* dg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 w = *reinterpret_cast<const float4*>(Wm + i * kP);
    const float4 q = *reinterpret_cast<const float4*>(Q + i * kP);
    for (int32_t e = gp[i]; e < gp[i + 1]; ++e) {
      const int64_t j = gi[e];
      const float4 r = *reinterpret_cast<const float4*>(R + j * kP);
      const float4 z = *reinterpret_cast<const float4*>(Z + j * kP);
      dg[e] = scale * (w.x * r.x + w.y * r.y + w.z * r.z + w.w * r.w + q.x * z.x + q.y * z.y + q.z * z.z + q.w * z.w);
    }
  }
}

// Gaussian probes from a counter hash (splitmix64) and the Box-Muller transform.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_probes(float* Z, int64_t count, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed * 0x9E3779B97F4A7C15ull + 2 * (uint64_t)i + 1);
    const uint64_t h2 = mix64(h1 + 0x632BE59BD9B4E019ull);
    const float u1 = ((float)(h1 >> 40) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = (float)(h2 >> 40) * (1.0f / 16777216.0f);
    Z[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  }
}

// --- backward of the heads ---------------------------------------------
// Per row (warp, lane = channel): diagonal -> dY[i][64]; off-diagonal edges
// -> dz_e (kept for the transposed gather), dY[i][0:32] (sum over the row's
// edges in order), and per-warp partial gradients of q, p3, p0, b_d written
// to `part` at [warp slot][4 x 32].
__global__ void k_edge_head_bwd(const float* __restrict__ Y, const int32_t* __restrict__ gp,
                                const int32_t* __restrict__ gi, const float* __restrict__ ga,
                                const float* __restrict__ params, int p3o, int p0o, int qo, int bdo,
                                const float* __restrict__ dg, int64_t n, float* dY, float* dz,
                                float* part) {
  const int lane = threadIdx.x & 31;
  const float p3 = params[p3o + lane], p0 = params[p0o + lane], q = params[qo + lane];
  const float bd = params[bdo];
  float gq = 0.f, gp3 = 0.f, gp0 = 0.f, gbd = 0.f;
  const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = wid; i < n; i += warps) {
    const float y1 = Y[i * kNH + lane];
    float dy1 = 0.f;
    float dyd = 0.f;
    for (int32_t e = gp[i]; e < gp[i + 1]; ++e) {
      const int32_t j = gi[e];
      const float d = dg[e];
      if (j == (int32_t)i) {
        const float tt = Y[i * kNH + 2 * kC] + bd;
        dyd = d * dsoftplus(tt);
        if (lane == 0) gbd += dyd;
      } else {
        const float pre = y1 + Y[(int64_t)j * kNH + kC + lane] + ga[e] * p3 + p0;
        const float z = fmaxf(pre, 0.f);
        gq += d * z;
        const float dzc = pre > 0.f ? d * q : 0.f;
        dz[(int64_t)e * kC + lane] = dzc;
        dy1 += dzc;
        gp3 += dzc * ga[e];
        gp0 += dzc;
      }
    }
    dY[i * kNH + lane] = dy1;
    if (lane < kNH - 2 * kC) dY[i * kNH + 2 * kC + lane] = lane == 0 ? dyd : 0.f;
  }
  float* pw = part + wid * (4 * kC);
  pw[lane] = gq;
  pw[kC + lane] = gp3;
  pw[2 * kC + lane] = gp0;
  pw[3 * kC + lane] = lane == 0 ? gbd : 0.f;
}

// dY[j][32:64] = sum over the edges (i, j), i > j, of dz_e (transposed gather, ascending i)
__global__ void k_gather_dy2(const int32_t* __restrict__ tp, const int32_t* __restrict__ ti,
                             const int32_t* __restrict__ tperm, const float* __restrict__ dz, int64_t n,
                             float* dY) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += warps) {
    float acc = 0.f;
    for (int32_t t = tp[j]; t < tp[j + 1]; ++t)
      if (ti[t] != (int32_t)j) acc += dz[(int64_t)tperm[t] * kC + lane];
    dY[j * kNH + kC + lane] = acc;
  }
}

// dH[i][k] = sum_o D[i][o] Wf[o][k]   (FP32, Wf = BF16-rounded weights [NO x KK])
template <int NO, int KK>
__global__ void __launch_bounds__(256) k_gemm_dgrad(const float* __restrict__ D, int ldd,
                                                    const float* __restrict__ Wf, int64_t n, float* out,
                                                    bool accumulate) {
  __shared__ float Ws[NO * KK];
  for (int i = threadIdx.x; i < NO * KK; i += blockDim.x) Ws[i] = Wf[i];
  __syncthreads();
  constexpr int TPR = KK;  // threads per row
  constexpr int RPB = 256 / TPR;
  const int k = threadIdx.x % TPR;
  for (int64_t i = (int64_t)blockIdx.x * RPB + threadIdx.x / TPR; i < n; i += (int64_t)gridDim.x * RPB) {
    float acc = 0.f;
    const float* d = D + i * ldd;
#pragma unroll 8
    for (int o = 0; o < NO; ++o) acc += d[o] * Ws[o * KK + k];
    if (accumulate) out[i * KK + k] += acc;
    else out[i * KK + k] = acc;
  }
}

// Weight gradients out[o][k] = sum_i D[i][o] X[i][k] over row chunks;
// one partial per block, reduced in block order by k_reduce_blocks.
template <int NO, int KK, int KX>
__global__ void __launch_bounds__(256) k_wgrad(const float* __restrict__ D, int ldd, const bf16* __restrict__ X,
                                               int64_t n, float* part) {
  constexpr int RB = 16;
  __shared__ float Ds[RB * NO];
  __shared__ float Xs[RB * KK];
  constexpr int OUT = NO * KK;
  constexpr int PER = (OUT + 255) / 256;
  float acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = 0.f;
  for (int64_t r0 = (int64_t)blockIdx.x * RB; r0 < n; r0 += (int64_t)gridDim.x * RB) {
    __syncthreads();
    for (int t = threadIdx.x; t < RB * NO; t += 256) {
      const int64_t r = r0 + t / NO;
      Ds[t] = r < n ? D[r * ldd + t % NO] : 0.f;
    }
    for (int t = threadIdx.x; t < RB * KK; t += 256) {
      const int64_t r = r0 + t / KK;
      Xs[t] = r < n ? __bfloat162float(X[r * KX + t % KK]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      const int idx = threadIdx.x + 256 * m;
      if (idx < OUT) {
        const int o = idx / KK, k = idx % KK;
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < RB; ++r) s += Ds[r * NO + o] * Xs[r * KK + k];
        acc[m] += s;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    const int idx = threadIdx.x + 256 * m;
    if (idx < OUT) part[(int64_t)blockIdx.x * OUT + idx] = acc[m];
  }
}

// out[j] (+)= sum_b part[b * stride + j] in block order
__global__ void k_reduce_blocks(const float* __restrict__ part, int nb, int stride, int count, float* out,
                                int out_stride_mult) {
  (void)out_stride_mult;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += part[(int64_t)b * stride + j];
    out[j] = s;
  }
}

// dpre = dH * (pre > 0); dS[:, 0:64] = dpre; db partials
__global__ void k_relu_bwd(const float* __restrict__ dH, const float* __restrict__ pre, int64_t n, float* dS) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * kH; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / kH;
    const int c = (int)(t % kH);
    dS[i * 2 * kH + c] = pre[t] > 0.f ? dH[t] : 0.f;
  }
}
// dS[j][64:128] = sum_i a^_ji dpre_i (A^ symmetric)
__global__ void k_agg_bwd(const int32_t* __restrict__ op, const int32_t* __restrict__ oi,
                          const float* __restrict__ ov, int64_t n, float* dS) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += warps) {
    float ax = 0.f, ay = 0.f;
    for (int32_t e = op[j]; e < op[j + 1]; ++e) {
      const float a = ov[e];
      const float2 d = *reinterpret_cast<const float2*>(dS + (int64_t)oi[e] * 2 * kH + 2 * lane);
      ax += a * d.x;
      ay += a * d.y;
    }
    *reinterpret_cast<float2*>(dS + j * 2 * kH + kH + 2 * lane) = make_float2(ax, ay);
  }
}
// column sums of dS[:, 0:64] (bias gradient), per-block partials
__global__ void k_colsum(const float* __restrict__ dS, int64_t n, float* part) {
  const int c = threadIdx.x & 63;
  const int rg = threadIdx.x >> 6;  // 4 row groups per block
  float s = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * 4 + rg; i < n; i += (int64_t)gridDim.x * 4) s += dS[i * 2 * kH + c];
  __shared__ float sh[256];
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < 64)
    part[(int64_t)blockIdx.x * 64 + c] = sh[c] + sh[64 + c] + sh[128 + c] + sh[192 + c];
}

// Adam step and the BF16 weight copies
__global__ void k_adam(float* p, const float* __restrict__ g, float* m, float* v, int count, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// combined layer weight [2kH x kpad] = [Ws; Wn] padded, and its FP32 copy
__global__ void k_pack_layer(const float* __restrict__ p, int ws, int wn, int kin, int kpad, bf16* wc, float* wcf) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * kH * kpad; t += gridDim.x * blockDim.x) {
    const int o = t / kpad, k = t % kpad;
    float w = 0.f;
    if (k < kin) w = o < kH ? p[ws + o * kin + k] : p[wn + (o - kH) * kin + k];
    const bf16 b = __float2bfloat16(w);
    wc[t] = b;
    wcf[t] = __bfloat162float(b);
  }
}
__global__ void k_pack_head(const float* __restrict__ p, int P1, int P2, int wd, bf16* wh, float* whf) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kNH * kH; t += gridDim.x * blockDim.x) {
    const int o = t / kH, k = t % kH;
    float w = 0.f;
    if (o < kC) w = p[P1 + o * kH + k];
    else if (o < 2 * kC) w = p[P2 + (o - kC) * kH + k];
    else if (o == 2 * kC) w = p[wd + k];
    const bf16 b = __float2bfloat16(w);
    wh[t] = b;
    whf[t] = __bfloat162float(b);
  }
}

// G values in the operator's precision: g_ij = d_i^-1/2 g^_ij
template <typename T>
__global__ void k_scale_g(const int32_t* __restrict__ gp, const float* __restrict__ g, const float* __restrict__ dis,
                          int64_t n, T* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    for (int32_t e = gp[i]; e < gp[i + 1]; ++e) out[e] = (T)((double)g[e] * (double)dis[i]);
}

// G^T values on the transposed pattern: entry k of G^T is entry perm[k] of G
template <typename T>
__global__ void k_gather_entries(const int32_t* __restrict__ perm, const T* __restrict__ src, int64_t m, T* out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = src[perm[k]];
}

// ============================================================ host side
int prep_graph(sx_ctx ctx, sx_gnn net, sx_op a, Graph** out) {
  for (auto& g : net->graphs)
    if (g.key == a->serial) { *out = &g; return SX_OK; }
  if (net->graphs.size() >= 64) {
    for (auto& g : net->graphs) graph_free(g);
    net->graphs.clear();
  }
  if (a->kind != SX_OP_CSR || a->nrows != a->ncols)
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: the network needs a square CSR matrix");
  if (!a->csr.has_sorted_indices || !a->csr.monotone)
    return set_error(SX_ERR_VALUE, "Value error: the network needs sorted column indices");
  Graph g;
  g.key = a->serial;
  g.n = a->nrows;
  const int64_t n = g.n;
  const int gr = vec_grid(ctx, n);
  int32_t *ocnt = nullptr, *gcnt = nullptr, *tcnt = nullptr;
  int* bad = nullptr;
  double* gidx = nullptr;
  int rc = SX_OK;
  do {
    const size_t nb = std::max<int64_t>(n, 1);
    if ((rc = dev_alloc((void**)&g.dis, nb * 4))) break;
    if ((rc = dev_alloc((void**)&bad, 16))) break;
    if ((rc = dev_alloc((void**)&ocnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&gcnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&tcnt, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.op, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.gp, (nb + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.tp, (nb + 1) * 4))) break;
    SX_CUDA(cudaMemsetAsync(bad, 0, 16, ctx->stream));
    if (a->dtype == SX_F64)
      k_dis<double><<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const double*)a->csr.vals, n, g.dis, bad);
    else
      k_dis<float><<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const float*)a->csr.vals, n, g.dis, bad);
    k_count_off_lower<<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, n, ocnt, gcnt);
    k_sym_pattern<<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, n, tcnt, bad + 1);
    ctx->launches += 3;
    if ((rc = exclusive_scan_i32(ctx, ocnt, n, g.op))) break;
    if ((rc = exclusive_scan_i32(ctx, gcnt, n, g.gp))) break;
    if ((rc = exclusive_scan_i32(ctx, tcnt, n, g.tp))) break;
    int hb[2] = {0, 0};
    int32_t noff = 0, ng = 0;
    SX_CUDA(cudaMemcpyAsync(hb, bad, 8, cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(&noff, g.op + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaMemcpyAsync(&ng, g.gp + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hb[0]) { rc = set_error(SX_ERR_VALUE, "Value error: the network needs a positive diagonal"); break; }
    const bool sym = hb[1] == 0;
    g.noff = noff;
    g.ng = ng;
    if ((rc = dev_alloc((void**)&g.oi, std::max(noff, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.ov, std::max(noff, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.gi, std::max(ng, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&g.ga, std::max(ng, 1) * 4))) break;
    if (!sym && (rc = dev_alloc((void**)&gidx, std::max(ng, 1) * 8))) break;
    if ((rc = dev_alloc((void**)&g.x0, nb * kK0 * sizeof(bf16)))) break;
    if (a->dtype == SX_F64)
      k_fill_graph<double><<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const double*)a->csr.vals, n,
                                                           g.dis, g.op, g.oi, g.ov, g.gp, g.gi, g.ga, g.x0, gidx);
    else
      k_fill_graph<float><<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const float*)a->csr.vals, n,
                                                          g.dis, g.op, g.oi, g.ov, g.gp, g.gi, g.ga, g.x0, gidx);
    ctx->launches++;
    if (sym) {
      // the transposed pattern read off A's upper triangle: no sort
      if ((rc = dev_alloc((void**)&g.ti, std::max(ng, 1) * 4))) break;
      if ((rc = dev_alloc((void**)&g.tperm, std::max(ng, 1) * 4))) break;
      k_gt_from_sym<<<gr, kBlock, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, n, g.gp, g.tp, g.ti, g.tperm);
      ctx->launches++;
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      break;
    }
    dev_free(g.tp);
    g.tp = nullptr;
    // any other pattern: the transpose with the entry permutation (exact
    // through FP64 values)
    sx_op s = new sx_op_s();
    s->kind = SX_OP_CSR;
    s->dtype = SX_F64;
    s->device = ctx->device;
    s->nrows = s->ncols = n;
    s->csr.nrows = s->csr.ncols = n;
    s->csr.nnz = ng;
    s->csr.indptr = g.gp;
    s->csr.indices = g.gi;
    s->csr.vals = gidx;
    sx_op t = nullptr;
    rc = csr_transpose_internal(ctx, s, &t, false);
    s->csr.indptr = nullptr; s->csr.indices = nullptr; s->csr.vals = nullptr;
    delete s;
    if (rc) break;
    g.tp = t->csr.indptr;
    g.ti = t->csr.indices;
    if ((rc = dev_alloc((void**)&g.tperm, std::max(ng, 1) * 4))) { destroy_op_internal(t); break; }
    k_perm_from_double<<<vec_grid(ctx, ng), kBlock, 0, ctx->stream>>>((const double*)t->csr.vals, ng, g.tperm);
    ctx->launches++;
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
    t->csr.indptr = nullptr; t->csr.indices = nullptr;
    destroy_op_internal(t);
  } while (0);
  dev_free(ocnt); dev_free(gcnt); dev_free(tcnt); dev_free(bad); dev_free(gidx);
  if (rc != SX_OK) { graph_free(g); return rc; }
  net->graphs.push_back(g);
  *out = &net->graphs.back();
  return SX_OK;
}

int acts_ensure(sx_gnn net, int64_t n, int64_t ng, int grid_warps) {
  Acts& A = net->acts;
  if (A.n >= n && A.ng >= ng) return SX_OK;
  for (int l = 1; l <= kL; ++l) dev_free(A.h[l]);
  for (int l = 0; l < kL; ++l) dev_free(A.pre[l]);
  dev_free(A.S); dev_free(A.Y); dev_free(A.dY); dev_free(A.dH); dev_free(A.dH2); dev_free(A.g); dev_free(A.dg);
  dev_free(A.dz); dev_free(A.Z); dev_free(A.Yp); dev_free(A.W); dev_free(A.V); dev_free(A.R); dev_free(A.Pp);
  dev_free(A.Q); dev_free(A.part); dev_free(A.dw);
  A = Acts{};
  const int64_t N = std::max<int64_t>(n, 1), G = std::max<int64_t>(ng, 1);
  for (int l = 1; l <= kL; ++l) SX_CHECK(dev_alloc((void**)&A.h[l], N * kH * sizeof(bf16)));
  for (int l = 0; l < kL; ++l) SX_CHECK(dev_alloc((void**)&A.pre[l], N * kH * 4));
  SX_CHECK(dev_alloc((void**)&A.S, N * 2 * kH * 4));
  SX_CHECK(dev_alloc((void**)&A.Y, N * kNH * 4));
  SX_CHECK(dev_alloc((void**)&A.dY, N * kNH * 4));
  SX_CHECK(dev_alloc((void**)&A.dH, N * kH * 4));
  SX_CHECK(dev_alloc((void**)&A.dH2, N * kH * 4));
  SX_CHECK(dev_alloc((void**)&A.g, G * 4));
  SX_CHECK(dev_alloc((void**)&A.dg, G * 4));
  SX_CHECK(dev_alloc((void**)&A.dz, G * kC * 4));
  float** probes[] = {&A.Z, &A.Yp, &A.W, &A.V, &A.R, &A.Pp, &A.Q};
  for (float** p : probes) SX_CHECK(dev_alloc((void**)p, N * kP * 4));
  A.part_floats = (size_t)std::max(grid_warps * 4 * kC, 2048 * 2 * kH * 64);
  SX_CHECK(dev_alloc((void**)&A.part, A.part_floats * 4));
  SX_CHECK(dev_alloc((void**)&A.dw, 2 * kH * kH * 4));
  A.n = n;
  A.ng = ng;
  return SX_OK;
}

void refresh_weights(sx_ctx ctx, sx_gnn net) {
  const Layout& L = net->L;
  for (int l = 0; l < kL; ++l) {
    const int kpad = l == 0 ? kK0 : kH;
    k_pack_layer<<<64, 256, 0, ctx->stream>>>(net->params, L.ws[l], L.wn[l], L.kin[l], kpad, net->wc[l], net->wcf[l]);
  }
  k_pack_head<<<32, 256, 0, ctx->stream>>>(net->params, L.P1, L.P2, L.wd, net->wh, net->whf);
  ctx->launches += kL + 1;
}

constexpr int kWarpGrid = 4096;   // blocks of 256 threads for warp-per-row kernels (8 warps each)

// keep_pre: store the pre-activations for a backward pass
int forward(sx_ctx ctx, sx_gnn net, const Graph& g, bool keep_pre) {
  Acts& A = net->acts;
  const int64_t n = g.n;
  const Layout& L = net->L;
  const unsigned gb = (unsigned)((n + kGemmRows - 1) / kGemmRows);
  const int wb = (int)std::min<int64_t>(kWarpGrid, (n + 7) / 8 + 1);
  A.h[0] = g.x0;
  for (int l = 0; l < kL; ++l) {
    if (n > 0) {
      if (l == 0) k_gemm_bf16<kK0, 2 * kH><<<gb, 128, 0, ctx->stream>>>(A.h[0], net->wc[0], A.S, n);
      else k_gemm_bf16<kH, 2 * kH><<<gb, 128, 0, ctx->stream>>>(A.h[l], net->wc[l], A.S, n);
      k_aggregate<<<wb, 256, 0, ctx->stream>>>(A.S, g.op, g.oi, g.ov, net->params + L.b[l], n,
                                               keep_pre ? A.pre[l] : nullptr, A.h[l + 1]);
      ctx->launches += 2;
    }
  }
  if (n > 0) {
    k_gemm_bf16<kH, kNH><<<gb, 128, 0, ctx->stream>>>(A.h[kL], net->wh, A.Y, n);
    k_edge_head<<<wb, 256, 0, ctx->stream>>>(A.Y, g.gp, g.gi, g.ga, net->params, L.p3, L.p0, L.q, L.bd, n, A.g);
    ctx->launches += 2;
  }
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

// loss (device scalar) and dg for the current edge values; Z already filled
int loss_and_dg(sx_ctx ctx, sx_gnn net, const Graph& g) {
  Acts& A = net->acts;
  const int64_t n = g.n;
  const int gr = vec_grid(ctx, n);
  k_spmm_g<<<gr, kBlock, 0, ctx->stream>>>(g.gp, g.gi, A.g, A.Z, n, A.Yp);
  k_spmm_a<<<gr, kBlock, 0, ctx->stream>>>(g.op, g.oi, g.ov, A.Yp, n, A.W);
  k_spmm_gt<<<gr, kBlock, 0, ctx->stream>>>(g.tp, g.ti, g.tperm, A.g, A.W, n, A.V);
  SX_CUDA(cudaMemsetAsync(net->counter, 0, 4, ctx->stream));
  k_resid_loss<<<vec_grid(ctx, n * kP), kBlock, 0, ctx->stream>>>(A.V, A.Z, n, A.R, A.part, net->counter, net->loss);
  k_spmm_g<<<gr, kBlock, 0, ctx->stream>>>(g.gp, g.gi, A.g, A.R, n, A.Pp);
  k_spmm_a<<<gr, kBlock, 0, ctx->stream>>>(g.op, g.oi, g.ov, A.Pp, n, A.Q);
  const float scale = 2.0f / (float)(kP * std::max<int64_t>(n, 1));
  k_sddmm<<<gr, kBlock, 0, ctx->stream>>>(g.gp, g.gi, A.W, A.R, A.Q, A.Z, n, scale, A.dg);
  ctx->launches += 7;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

int wgrad(sx_ctx ctx, sx_gnn net, const float* D, int ldd, int no, const bf16* X, int kx, int kk, int64_t n,
          float* out_o_k) {
  Acts& A = net->acts;
  const int nb = (int)std::min<int64_t>(2048, std::max<int64_t>((n + 15) / 16, 1));
  if (no == 2 * kH && kk == kF0)
    k_wgrad<2 * kH, kF0, kK0><<<nb, 256, 0, ctx->stream>>>(D, ldd, X, n, A.part);
  else if (no == 2 * kH && kk == kH)
    k_wgrad<2 * kH, kH, kH><<<nb, 256, 0, ctx->stream>>>(D, ldd, X, n, A.part);
  else if (no == kNH && kk == kH)
    k_wgrad<kNH, kH, kH><<<nb, 256, 0, ctx->stream>>>(D, ldd, X, n, A.part);
  else
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: weight-gradient shape");
  k_reduce_blocks<<<64, 256, 0, ctx->stream>>>(A.part, nb, no * kk, no * kk, out_o_k, 0);
  ctx->launches += 2;
  return SX_OK;
}

__global__ void k_scatter_layer_grad(const float* __restrict__ dwc, int kin, float* grad, int ws, int wn) {
  // dwc is [2kH x kin]: rows 0..63 -> Ws, 64..127 -> Wn
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * kH * kin; t += gridDim.x * blockDim.x) {
    const int o = t / kin, k = t % kin;
    if (o < kH) grad[ws + o * kin + k] = dwc[t];
    else grad[wn + (o - kH) * kin + k] = dwc[t];
  }
}
__global__ void k_scatter_head_grad(const float* __restrict__ dwh, float* grad, int P1, int P2, int wd) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kNH * kH; t += gridDim.x * blockDim.x) {
    const int o = t / kH, k = t % kH;
    if (o < kC) grad[P1 + o * kH + k] = dwh[t];
    else if (o < 2 * kC) grad[P2 + (o - kC) * kH + k] = dwh[t];
    else if (o == 2 * kC) grad[wd + k] = dwh[t];
  }
}
// small head parameters from the per-warp partials [nw x 4 x kC]
__global__ void k_reduce_head_small(const float* __restrict__ part, int nw, float* grad, int q, int p3, int p0,
                                    int bd) {
  const int t = threadIdx.x;  // 0 .. 4*kC-1
  if (t >= 4 * kC) return;
  float s = 0.f;
  for (int w = 0; w < nw; ++w) s += part[(int64_t)w * 4 * kC + t];
  const int which = t / kC, c = t % kC;
  if (which == 0) grad[q + c] = s;
  else if (which == 1) grad[p3 + c] = s;
  else if (which == 2) grad[p0 + c] = s;
  else if (c == 0) grad[bd] = s;
}

int backward(sx_ctx ctx, sx_gnn net, const Graph& g) {
  Acts& A = net->acts;
  const Layout& L = net->L;
  const int64_t n = g.n;
  float* dw = A.dw;
  SX_CUDA(cudaMemsetAsync(net->grad, 0, (size_t)L.total * 4, ctx->stream));
  if (n == 0) return SX_OK;
  const int wb = (int)std::min<int64_t>(kWarpGrid, (n + 7) / 8 + 1);
  // heads
  k_edge_head_bwd<<<wb, 256, 0, ctx->stream>>>(A.Y, g.gp, g.gi, g.ga, net->params, L.p3, L.p0, L.q, L.bd, A.dg, n,
                                               A.dY, A.dz, A.part);
  k_reduce_head_small<<<1, 4 * kC, 0, ctx->stream>>>(A.part, wb * 8, net->grad, L.q, L.p3, L.p0, L.bd);
  k_gather_dy2<<<wb, 256, 0, ctx->stream>>>(g.tp, g.ti, g.tperm, A.dz, n, A.dY);
  ctx->launches += 3;
  SX_CHECK(wgrad(ctx, net, A.dY, kNH, kNH, A.h[kL], kH, kH, n, dw));
  k_scatter_head_grad<<<32, 256, 0, ctx->stream>>>(dw, net->grad, L.P1, L.P2, L.wd);
  k_gemm_dgrad<kNH, kH><<<2048, 256, 0, ctx->stream>>>(A.dY, kNH, net->whf, n, A.dH, false);
  ctx->launches += 2;
  // layers, last to first
  for (int l = kL - 1; l >= 0; --l) {
    k_relu_bwd<<<vec_grid(ctx, n * kH), kBlock, 0, ctx->stream>>>(A.dH, A.pre[l], n, A.S);
    k_agg_bwd<<<wb, 256, 0, ctx->stream>>>(g.op, g.oi, g.ov, n, A.S);
    const int cb = (int)std::min<int64_t>(1024, (n + 3) / 4);
    k_colsum<<<cb, 256, 0, ctx->stream>>>(A.S, n, A.part);
    k_reduce_blocks<<<1, 64, 0, ctx->stream>>>(A.part, cb, 64, 64, net->grad + L.b[l], 0);
    ctx->launches += 4;
    const int kin = L.kin[l];
    if (l == 0) SX_CHECK(wgrad(ctx, net, A.S, 2 * kH, 2 * kH, A.h[0], kK0, kF0, n, dw));
    else SX_CHECK(wgrad(ctx, net, A.S, 2 * kH, 2 * kH, A.h[l], kH, kH, n, dw));
    k_scatter_layer_grad<<<32, 256, 0, ctx->stream>>>(dw, kin, net->grad, L.ws[l], L.wn[l]);
    ctx->launches++;
    if (l > 0) {
      k_gemm_dgrad<2 * kH, kH><<<2048, 256, 0, ctx->stream>>>(A.S, 2 * kH, net->wcf[l], n, A.dH2, false);
      ctx->launches++;
      std::swap(A.dH, A.dH2);
    }
  }
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

void init_params(std::vector<float>& p, const Layout& L, uint64_t seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<float> U(-1.f, 1.f);
  p.assign(L.total, 0.f);
  for (int l = 0; l < kL; ++l) {
    const float s = std::sqrt(1.0f / (float)L.kin[l]);
    for (int i = 0; i < kH * L.kin[l]; ++i) {
      p[L.ws[l] + i] = s * U(rng);
      p[L.wn[l] + i] = s * U(rng);
    }
  }
  const float s = std::sqrt(1.0f / (float)kH);
  for (int i = 0; i < kC * kH; ++i) {
    p[L.P1 + i] = s * U(rng);
    p[L.P2 + i] = s * U(rng);
  }
  for (int c = 0; c < kC; ++c) {
    p[L.p3 + c] = U(rng);
    p[L.p0 + c] = 0.1f * U(rng);
    p[L.q + c] = 0.01f * U(rng);
  }
  for (int k = 0; k < kH; ++k) p[L.wd + k] = 0.01f * U(rng);
  p[L.bd] = 0.5413248546129181f;  // softplus^-1(1): G^ starts at the identity (Jacobi)
}

}  // namespace gnn
}  // namespace sx

using namespace sx;
using namespace sx::gnn;

extern "C" {

uint64_t sx_gnn_num_params(void) { return (uint64_t)layout().total; }

int sx_gnn_create(sx_ctx ctx, const float* params, uint64_t seed, sx_gnn* out) {
  if (!ctx || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  sx_gnn net = new sx_gnn_s();
  net->device = ctx->device;
  net->L = layout();
  const int P = net->L.total;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&net->params, P * 4))) break;
    if ((rc = dev_alloc((void**)&net->grad, P * 4))) break;
    if ((rc = dev_alloc((void**)&net->m, P * 4))) break;
    if ((rc = dev_alloc((void**)&net->v, P * 4))) break;
    for (int l = 0; l < kL; ++l) {
      const int kpad = l == 0 ? kK0 : kH;
      if ((rc = dev_alloc((void**)&net->wc[l], 2 * kH * kpad * sizeof(bf16)))) break;
      if ((rc = dev_alloc((void**)&net->wcf[l], 2 * kH * kpad * 4))) break;
    }
    if (rc) break;
    if ((rc = dev_alloc((void**)&net->wh, kNH * kH * sizeof(bf16)))) break;
    if ((rc = dev_alloc((void**)&net->whf, kNH * kH * 4))) break;
    if ((rc = dev_alloc((void**)&net->loss, 16))) break;
    if ((rc = dev_alloc((void**)&net->counter, 16))) break;
    std::vector<float> h;
    if (params) h.assign(params, params + P);
    else init_params(h, net->L, seed);
    SX_CUDA(cudaMemcpy(net->params, h.data(), P * 4, cudaMemcpyHostToDevice));
    SX_CUDA(cudaMemset(net->m, 0, P * 4));
    SX_CUDA(cudaMemset(net->v, 0, P * 4));
    SX_CUDA(cudaMemset(net->counter, 0, 16));
    refresh_weights(ctx, net);
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
  } while (0);
  if (rc) {
    sx_gnn_destroy(net);
    return rc;
  }
  *out = net;
  return clear_error();
}

int sx_gnn_destroy(sx_gnn net) {
  if (!net) return SX_OK;
  cudaSetDevice(net->device);
  cudaDeviceSynchronize();
  dev_free(net->params); dev_free(net->grad); dev_free(net->m); dev_free(net->v);
  for (int l = 0; l < kL; ++l) { dev_free(net->wc[l]); dev_free(net->wcf[l]); }
  dev_free(net->wh); dev_free(net->whf); dev_free(net->loss); dev_free(net->counter);
  for (auto& g : net->graphs) graph_free(g);
  Acts& A = net->acts;
  for (int l = 1; l <= kL; ++l) dev_free(A.h[l]);
  for (int l = 0; l < kL; ++l) dev_free(A.pre[l]);
  dev_free(A.S); dev_free(A.Y); dev_free(A.dY); dev_free(A.dH); dev_free(A.dH2); dev_free(A.g); dev_free(A.dg);
  dev_free(A.dz); dev_free(A.Z); dev_free(A.Yp); dev_free(A.W); dev_free(A.V); dev_free(A.R); dev_free(A.Pp);
  dev_free(A.Q); dev_free(A.part); dev_free(A.dw);
  delete net;
  return SX_OK;
}

int sx_gnn_get_params(sx_ctx ctx, sx_gnn net, float* out) {
  if (!ctx || !net || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CUDA(cudaMemcpyAsync(out, net->params, (size_t)net->L.total * 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return SX_OK;
}

int sx_gnn_set_params(sx_ctx ctx, sx_gnn net, const float* in) {
  if (!ctx || !net || !in) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CUDA(cudaMemcpyAsync(net->params, in, (size_t)net->L.total * 4, cudaMemcpyHostToDevice, ctx->stream));
  refresh_weights(ctx, net);
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return SX_OK;
}

// Loss and gradient (no update).  probes: host n x 4 row-major, or NULL for
// seeded Gaussian probes.  grad_out: host, sx_gnn_num_params() floats (may be NULL).
int sx_gnn_loss_grad(sx_ctx ctx, sx_gnn net, sx_op a, const float* probes, uint64_t seed, float* loss_out,
                     float* grad_out) {
  if (!ctx || !net || !a) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CUDA(cudaSetDevice(ctx->device));
  Graph* g = nullptr;
  SX_CHECK(prep_graph(ctx, net, a, &g));
  SX_CHECK(acts_ensure(net, g->n, g->ng, kWarpGrid * 8));
  SX_CHECK(forward(ctx, net, *g, true));
  if (probes) SX_CUDA(cudaMemcpyAsync(net->acts.Z, probes, g->n * kP * 4, cudaMemcpyHostToDevice, ctx->stream));
  else {
    k_probes<<<vec_grid(ctx, g->n * kP), kBlock, 0, ctx->stream>>>(net->acts.Z, g->n * kP, seed);
    ctx->launches++;
  }
  SX_CHECK(loss_and_dg(ctx, net, *g));
  SX_CHECK(backward(ctx, net, *g));
  float l = 0.f;
  SX_CUDA(cudaMemcpyAsync(&l, net->loss, 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (grad_out)
    SX_CUDA(cudaMemcpyAsync(grad_out, net->grad, (size_t)net->L.total * 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (loss_out) *loss_out = l;
  return clear_error();
}

// One Adam step on the probe loss of matrix a (seeded probes).
int sx_gnn_train_step(sx_ctx ctx, sx_gnn net, sx_op a, uint64_t seed, float lr, float* loss_out) {
  SX_CHECK(sx_gnn_loss_grad(ctx, net, a, nullptr, seed, loss_out, nullptr));
  net->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)net->step), c2 = 1.f - std::pow(b2, (float)net->step);
  k_adam<<<64, 256, 0, ctx->stream>>>(net->params, net->grad, net->m, net->v, net->L.total, lr, b1, b2, 1e-8f, c1, c2);
  ctx->launches++;
  refresh_weights(ctx, net);
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return clear_error();
}

// Edge values g^ of the current network for matrix a (host copy; ng entries
// in G-pattern order: each row's strictly lower entries by column, then the
// diagonal).  ng_out receives the count; g_out may be NULL.
int sx_gnn_edge_values(sx_ctx ctx, sx_gnn net, sx_op a, float* g_out, uint64_t* ng_out) {
  if (!ctx || !net || !a) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  SX_CUDA(cudaSetDevice(ctx->device));
  Graph* g = nullptr;
  SX_CHECK(prep_graph(ctx, net, a, &g));
  SX_CHECK(acts_ensure(net, g->n, g->ng, kWarpGrid * 8));
  SX_CHECK(forward(ctx, net, *g, false));
  if (ng_out) *ng_out = (uint64_t)g->ng;
  if (g_out) SX_CUDA(cudaMemcpyAsync(g_out, net->acts.g, g->ng * 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return clear_error();
}

// M^-1 = G G^T with G = D^-1/2 G^ predicted for matrix a (dtype of a).
int sx_precond_learned(sx_ctx ctx, sx_op a, sx_gnn net, sx_op* out) {
  if (!ctx || !a || !net || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  Graph* g = nullptr;
  const size_t cached = net->graphs.size();
  SX_CHECK(prep_graph(ctx, net, a, &g));
  // a matrix seen only here is not kept: its prepared graph is dropped at
  // the end (training keeps the graphs of its problems)
  const bool fresh = net->graphs.size() > cached;
  auto drop_fresh = [&]() {
    if (fresh && !net->graphs.empty()) {
      cudaStreamSynchronize(ctx->stream);
      graph_free(net->graphs.back());
      net->graphs.pop_back();
    }
  };
  int frc = acts_ensure(net, g->n, g->ng, kWarpGrid * 8);
  if (frc == SX_OK) frc = forward(ctx, net, *g, false);
  if (frc != SX_OK) { drop_fresh(); return frc; }
  const int64_t n = g->n;
  const size_t w = elt_size(a->dtype);
  void* gv = nullptr;
  int rc = SX_OK;
  do {
    // G = D^-1/2 G^ on the network's pattern (rows sorted: the strictly
    // lower entries by column, then the diagonal), adopted as a CSR
    // operator without a round trip through the validating constructors
    if ((rc = dev_alloc(&gv, std::max<int64_t>(g->ng, 1) * w))) break;
    const int gr = vec_grid(ctx, n);
    if (a->dtype == SX_F64) k_scale_g<double><<<gr, kBlock, 0, ctx->stream>>>(g->gp, net->acts.g, g->dis, n, (double*)gv);
    else k_scale_g<float><<<gr, kBlock, 0, ctx->stream>>>(g->gp, net->acts.g, g->dis, n, (float*)gv);
    ctx->launches++;
    DevCsr c;
    c.nrows = c.ncols = n;
    c.nnz = g->ng;
    c.vals = gv;
    gv = nullptr;
    if ((rc = dev_alloc((void**)&c.indptr, (n + 1) * 4)) == SX_OK &&
        (rc = dev_alloc((void**)&c.indices, std::max<int64_t>(g->ng, 1) * 4)) == SX_OK) {
      cudaMemcpyAsync(c.indptr, g->gp, (n + 1) * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      if (g->ng > 0) cudaMemcpyAsync(c.indices, g->gi, g->ng * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      rc = csr_finalize_stats(ctx, c, (int)w);
    }
    // G^T on the transposed pattern the graph already holds: a gather of
    // G's values instead of a second transpose (the same arrays: the
    // graph's transpose is the counting sort of G's pattern)
    DevCsr t;
    t.nrows = t.ncols = n;
    t.nnz = g->ng;
    if (rc == SX_OK && (rc = dev_alloc((void**)&t.indptr, (n + 1) * 4)) == SX_OK &&
        (rc = dev_alloc((void**)&t.indices, std::max<int64_t>(g->ng, 1) * 4)) == SX_OK &&
        (rc = dev_alloc(&t.vals, std::max<int64_t>(g->ng, 1) * w)) == SX_OK) {
      cudaMemcpyAsync(t.indptr, g->tp, (n + 1) * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      if (g->ng > 0) {
        cudaMemcpyAsync(t.indices, g->ti, g->ng * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        const int ge = vec_grid(ctx, g->ng);
        if (a->dtype == SX_F64)
          k_gather_entries<double><<<ge, kBlock, 0, ctx->stream>>>(g->tperm, (const double*)c.vals, g->ng,
                                                                   (double*)t.vals);
        else
          k_gather_entries<float><<<ge, kBlock, 0, ctx->stream>>>(g->tperm, (const float*)c.vals, g->ng,
                                                                  (float*)t.vals);
        ctx->launches++;
      }
      rc = csr_finalize_stats(ctx, t, (int)w);
    }
    if (rc != SX_OK) {
      destroy_op_internal(csr_op_adopt(ctx, a->dtype, c));  // frees the arrays
      destroy_op_internal(csr_op_adopt(ctx, a->dtype, t));
      break;
    }
    rc = fsai_adopt(ctx, csr_op_adopt(ctx, a->dtype, c), out, csr_op_adopt(ctx, a->dtype, t));
    // the factor's values in FP16 for the solvers (the network's output is
    // already limited by its BF16 weights); FP32 stays for exact applies
    if (rc == SX_OK && a->dtype == SX_F32) {
      rc = csr_make_half(ctx, (*out)->csr);
      if (rc == SX_OK) rc = csr_make_half(ctx, (*out)->transpose->csr);
      if (rc == SX_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        rc = set_error(SX_ERR_CUDA, "CUDA error in the FP16 factor copy");
      if (rc != SX_OK) { destroy_op_internal(*out); *out = nullptr; }
    }
  } while (0);
  dev_free(gv);
  drop_fresh();
  return rc == SX_OK ? clear_error() : rc;
}

}  // extern "C"
