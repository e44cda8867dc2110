// Device building blocks shared by the kernels of the sparse library:
//  - deterministic grid reductions: per-block partials, the last block to
//    finish sums them in a fixed order and runs a finalize step;
//  - the CSR "stream" SpMV: a block owns a run of consecutive rows, streams
//    their nonzeros through shared memory in coalesced tiles, and each thread
//    sums its own row sequentially in storage order (the reference's order,
//    so the result is bit-identical to `sum = sum + a*x` per row);
//  - a grid-stride elementwise kernel with the same reduction tail.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace sx {

constexpr int kBlock = 256;        // threads per block of every kernel here
constexpr int kWarps = kBlock / 32;

template <typename T>
struct Acc3 {
  T a, b, c;
};

// Products and sums with rounding made explicit, so that the compiler never
// contracts a*b+c into one FMA: the reference rounds both operations.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of three values; the result is valid in every thread.
template <typename T>
__device__ __forceinline__ Acc3<T> block_sum3(Acc3<T> v) {
  __shared__ T sh[3][kWarps];
  __shared__ T out[3];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v.a = warp_sum(v.a);
  v.b = warp_sum(v.b);
  v.c = warp_sum(v.c);
  if (lane == 0) { sh[0][w] = v.a; sh[1][w] = v.b; sh[2][w] = v.c; }
  __syncthreads();
  if (w == 0) {
    T a = lane < kWarps ? sh[0][lane] : T(0);
    T b = lane < kWarps ? sh[1][lane] : T(0);
    T c = lane < kWarps ? sh[2][lane] : T(0);
    a = warp_sum(a); b = warp_sum(b); c = warp_sum(c);
    if (lane == 0) { out[0] = a; out[1] = b; out[2] = c; }
  }
  __syncthreads();
  Acc3<T> r{out[0], out[1], out[2]};
  __syncthreads();
  return r;
}

// Grid reduction tail.  Every block calls this once with its thread-local
// partials.  Returns true in the block that finished last; there, `tot`
// holds the grid totals (in every thread).  The counter is left at zero for
// the next launch.  The totals do not depend on which block finishes last.
template <typename T>
__device__ __forceinline__ bool grid_reduce3(Acc3<T> v, T* partials, unsigned int* counter,
                                             Acc3<T>& tot) {
  __shared__ bool s_last;
  Acc3<T> b = block_sum3(v);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x + 0] = b.a;
    partials[3 * blockIdx.x + 1] = b.b;
    partials[3 * blockIdx.x + 2] = b.c;
    __threadfence();
    unsigned int t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  Acc3<T> s{T(0), T(0), T(0)};
  for (unsigned int j = threadIdx.x; j < gridDim.x; j += kBlock) {
    s.a += __ldcg(partials + 3 * j + 0);
    s.b += __ldcg(partials + 3 * j + 1);
    s.c += __ldcg(partials + 3 * j + 2);
  }
  tot = block_sum3(s);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// --------------------------------------------------------------- SpMV
// Epilogue interface (all __device__):
//   bool skip() const                        -> whole launch is a no-op
//   T out(int64_t row, T ax) const           -> value stored to y[row]
//   void acc(int64_t row, T y, Acc3<T>& a)   -> per-row reduction terms (from
//                                               the value y, never from memory
//                                               at y[row])
//   static constexpr bool kReduce            -> run the grid reduction
//   void finish(const Acc3<T>& tot)          -> thread 0 of the last block
template <typename T>
struct Vec4 {
  T v[4];
};

// 4 consecutive values with 128-bit loads (two for double)
__device__ __forceinline__ Vec4<float> ld4(const float* p) {
  float4 a = __ldcs(reinterpret_cast<const float4*>(p));
  return Vec4<float>{{a.x, a.y, a.z, a.w}};
}
__device__ __forceinline__ Vec4<double> ld4(const double* p) {
  double2 a = __ldcs(reinterpret_cast<const double2*>(p));
  double2 b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
  return Vec4<double>{{a.x, a.y, b.x, b.y}};
}
// 4 consecutive FP16 values (one 64-bit load), widened to FP32
__device__ __forceinline__ Vec4<float> ld4(const __half* p) {
  const uint2 u = __ldcs(reinterpret_cast<const uint2*>(p));
  const __half2 a = *reinterpret_cast<const __half2*>(&u.x);
  const __half2 b = *reinterpret_cast<const __half2*>(&u.y);
  const float2 fa = __half22float2(a), fb = __half22float2(b);
  return Vec4<float>{{fa.x, fa.y, fb.x, fb.y}};
}
template <typename T>
struct DiaVec {
  static constexpr int kVec = 16 / (int)sizeof(T);
};
__device__ __forceinline__ void vload(const float* p, float (&o)[4]) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}
__device__ __forceinline__ void vload(const double* p, double (&o)[2]) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  o[0] = a.x; o[1] = a.y;
}
__device__ __forceinline__ void vload(const __half* p, float (&o)[4]) {
  const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
  const float2 fa = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
  const float2 fb = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
  o[0] = fa.x; o[1] = fa.y; o[2] = fb.x; o[3] = fb.y;
}

__device__ __forceinline__ float to_val(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_val(float v) { return v; }
__device__ __forceinline__ double to_val(double v) { return v; }
__device__ __forceinline__ int4 ld4i(const int32_t* p) {
  return __ldcs(reinterpret_cast<const int4*>(p));
}

template <typename T, int ITEMS, class Epi, bool FMA = false>
__global__ void __launch_bounds__(kBlock) spmv_stream_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const T* __restrict__ vals, const T* __restrict__ x, T* __restrict__ y, int64_t nrows,
    T* partials, unsigned int* counter, Epi epi) {
  if (epi.skip()) return;
  // A tile covers TILE nonzeros starting at a multiple of 4, so every thread
  // moves 4 consecutive columns and values with 128-bit loads; the products
  // go to shared memory and each thread then sums its own row in order.
  constexpr int CH = ITEMS / 4;
  constexpr int TILE = kBlock * ITEMS;
  // FMA mode keeps value and x in shared memory and sums with fused
  // multiply-adds in the same order (one rounding per term instead of two)
  __shared__ int32_t s_ptr[kBlock + 1];
  __shared__ T s_prod[TILE];
  __shared__ T s_x[FMA ? TILE : 1];
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * kBlock;
  const int nr = (int)min((int64_t)kBlock, nrows - r0);
  if (tid <= nr) s_ptr[tid] = indptr[r0 + tid];
  if (tid == 0 && nr == kBlock) s_ptr[kBlock] = indptr[r0 + kBlock];
  __syncthreads();
  const int32_t s = s_ptr[0], e = s_ptr[nr];
  int32_t my_s = 0, my_e = 0;
  if (tid < nr) { my_s = s_ptr[tid]; my_e = s_ptr[tid + 1]; }
  T acc = T(0);
  auto put = [&](int32_t slot, T v, T xv) {
    if constexpr (FMA) { s_prod[slot] = v; s_x[slot] = xv; }
    else s_prod[slot] = mul_rn(v, xv);
  };
  for (int32_t base = s & ~3; base < e; base += TILE) {
    const int32_t tend = min(e, base + TILE);
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int32_t k0 = base + (c * kBlock + tid) * 4;
      if (k0 < tend) {
        // k0 + 3 < e implies an in-bounds vector (e <= nnz)
        if (k0 + 3 < e) {
          const int4 ci = ld4i(indices + k0);
          const Vec4<T> cv = ld4(vals + k0);
          const int cc[4] = {ci.x, ci.y, ci.z, ci.w};
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (k0 + q >= s) put(k0 + q - base, cv.v[q], __ldg(x + cc[q]));
        } else {
          for (int q = 0; q < 4; ++q) {
            const int32_t k = k0 + q;
            if (k >= s && k < e) put(k - base, vals[k], __ldg(x + indices[k]));
          }
        }
      }
    }
    __syncthreads();
    if (tid < nr) {
      const int32_t lo = max(my_s, base), hi = min(my_e, tend);
      if constexpr (FMA) {
        for (int32_t k = lo; k < hi; ++k) acc = fma(s_prod[k - base], s_x[k - base], acc);
      } else {
        for (int32_t k = lo; k < hi; ++k) acc = add_rn(acc, s_prod[k - base]);
      }
    }
    __syncthreads();
  }
  Acc3<T> a{T(0), T(0), T(0)};
  if (tid < nr) {
    const int64_t row = r0 + tid;
    const T v = epi.out(row, acc);
    y[row] = v;
    epi.acc(row, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && tid == 0) epi.finish(tot);
  }
}

// Pipelined persistent variant for matrices whose 256-row chunks each fit
// one tile (chunk nnz + 3 <= 256 * ITEMS).  A block walks chunks
// c, c + gridDim.x, ...; the row pointers and the 128-bit column/value loads
// of the next chunk are issued while the current chunk gathers x and sums
// its rows, so two chunks per block are in flight.  Per-row order and
// rounding are those of spmv_stream_kernel (bit-identical results).
// C16: columns come from the compressed copy, col = chunk_base[chunk] +
// col16[k] (16-bit offsets, 2 bytes per entry instead of 4).  MINB asks the
// compiler for that many resident blocks per SM (a register budget).  V is
// the storage type of the values (FP16 for the learned factor, widened to T).
// Gather supplies the vector entries (x[col], or a vector formed on the fly).
// x[col]: the plain gather of the SpMV kernels
template <typename T>
struct GatherPlain {
  __device__ __forceinline__ T operator()(const T* __restrict__ x, int col) const { return __ldg(x + col); }
  // 16 bytes at an aligned column (the diagonal-layout kernel)
  template <int VEC>
  __device__ __forceinline__ void vec(const T* __restrict__ x, int col, T (&o)[VEC]) const { vload(x + col, o); }
};

template <typename T, int ITEMS, class Epi, bool FMA = false, bool C16 = false, int MINB = 1, typename V = T,
          class Gather = GatherPlain<T>>
__global__ void __launch_bounds__(kBlock, MINB) spmv_pipe_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const V* __restrict__ vals, const T* __restrict__ x, T* __restrict__ y, int64_t nrows,
    int64_t nchunks, T* partials, unsigned int* counter, Epi epi,
    const uint16_t* __restrict__ col16 = nullptr, const int32_t* __restrict__ chunk_base = nullptr,
    Gather gat = Gather{}) {
  if (epi.skip()) return;
  constexpr int CH = ITEMS / 4;
  constexpr int TILE = kBlock * ITEMS;
  __shared__ T s_prod[TILE];
  __shared__ T s_x[FMA ? TILE : 1];
  const int tid = threadIdx.x;
  // registers of the chunk in flight
  int32_t cs = 0, ce = 0, ms = 0, me = 0;
  int4 ci[CH];
  Vec4<T> cv[CH];
  // cb: the chunk's column base (C16 only)
  auto load_meta = [&](int64_t ch, int32_t& s0, int32_t& e0, int32_t& m0, int32_t& m1, int32_t& cb) {
    const int64_t r0 = ch * kBlock;
    const int nr = (int)min((int64_t)kBlock, nrows - r0);
    s0 = __ldg(indptr + r0);
    e0 = __ldg(indptr + r0 + nr);
    if (tid < nr) { m0 = __ldg(indptr + r0 + tid); m1 = __ldg(indptr + r0 + tid + 1); }
    else { m0 = 0; m1 = 0; }
    if constexpr (C16) cb = __ldg(chunk_base + ch);
  };
  auto load_data = [&](int32_t s0, int32_t e0, int32_t cb, int4* di, Vec4<T>* dv) {
    const int32_t base = s0 & ~3;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int32_t k0 = base + (c * kBlock + tid) * 4;
      if (k0 + 3 < e0) {
        if constexpr (C16) {
          const uint2 o = __ldcs(reinterpret_cast<const uint2*>(col16 + k0));
          di[c] = make_int4(cb + (int)(o.x & 0xffffu), cb + (int)(o.x >> 16), cb + (int)(o.y & 0xffffu),
                            cb + (int)(o.y >> 16));
        } else {
          di[c] = ld4i(indices + k0);
        }
        dv[c] = ld4(vals + k0);
      } else {
        int cc[4];
        T vv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int32_t k = k0 + q;
          const bool in = k < e0;
          if constexpr (C16) cc[q] = in ? cb + (int)col16[k] : 0;
          else cc[q] = in ? indices[k] : 0;
          vv[q] = in ? (T)to_val(vals[k]) : T(0);
        }
        di[c] = make_int4(cc[0], cc[1], cc[2], cc[3]);
        dv[c] = Vec4<T>{{vv[0], vv[1], vv[2], vv[3]}};
      }
    }
  };
  Acc3<T> a{T(0), T(0), T(0)};
  int64_t ch = blockIdx.x;
  // row pointers run two chunks ahead, columns and values one chunk ahead:
  // the next chunk's loads are in flight while this chunk is summed
  int32_t ns = 0, ne = 0, nms = 0, nme = 0, cbc = 0, cbn = 0;
  if (ch < nchunks) {
    load_meta(ch, cs, ce, ms, me, cbc);
    load_data(cs, ce, cbc, ci, cv);
    if (ch + gridDim.x < nchunks) load_meta(ch + gridDim.x, ns, ne, nms, nme, cbn);
  }
  while (ch < nchunks) {
    const int64_t nxt = ch + gridDim.x;
    const int32_t base = cs & ~3;
    // products of the current chunk into shared memory
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int32_t k0 = base + (c * kBlock + tid) * 4;
      const int cc[4] = {ci[c].x, ci[c].y, ci[c].z, ci[c].w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int32_t k = k0 + q;
        if (k >= cs && k < ce) {
          const T xv = gat(x, cc[q]);
          if constexpr (FMA) { s_prod[k - base] = cv[c].v[q]; s_x[k - base] = xv; }
          else s_prod[k - base] = mul_rn(cv[c].v[q], xv);
        }
      }
    }
    // columns and values of the next chunk, row pointers of the one after
    // (the registers of this chunk are free once its products are stored)
    int32_t n2s = 0, n2e = 0, n2ms = 0, n2me = 0, cb2 = 0;
    if (nxt < nchunks) {
      load_data(ns, ne, cbn, ci, cv);
      if (nxt + gridDim.x < nchunks) load_meta(nxt + gridDim.x, n2s, n2e, n2ms, n2me, cb2);
    }
    __syncthreads();
    const int64_t row = ch * kBlock + tid;
    if (row < nrows) {
      T acc = T(0);
      if constexpr (FMA) {
        for (int32_t k = ms; k < me; ++k) acc = fma(s_prod[k - base], s_x[k - base], acc);
      } else {
        for (int32_t k = ms; k < me; ++k) acc = add_rn(acc, s_prod[k - base]);
      }
      const T v = epi.out(row, acc);
      y[row] = v;
      epi.acc(row, v, a);
    }
    __syncthreads();
    cs = ns; ce = ne; ms = nms; me = nme;
    ns = n2s; ne = n2e; nms = n2ms; nme = n2me; cbn = cb2;
    ch = nxt;
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && tid == 0) epi.finish(tot);
  }
}

// Rows whose end precedes their start (accepted by CsrArray::new) are
// empty; this one-thread-per-row kernel serves such irregular matrices.
template <typename T, class Epi>
__global__ void __launch_bounds__(kBlock) spmv_rowseq_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const T* __restrict__ vals, const T* __restrict__ x, T* __restrict__ y, int64_t nrows,
    T* partials, unsigned int* counter, Epi epi) {
  if (epi.skip()) return;
  const int64_t row = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  Acc3<T> a{T(0), T(0), T(0)};
  if (row < nrows) {
    T acc = T(0);
    for (int32_t k = indptr[row]; k < indptr[row + 1]; ++k)
      acc = add_rn(acc, mul_rn(vals[k], __ldg(x + indices[k])));
    const T v = epi.out(row, acc);
    y[row] = v;
    epi.acc(row, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

// plain (cacheable) 4-wide loads and stores for solver vectors, which the
// next kernel reads again
__device__ __forceinline__ Vec4<float> ldv4(const float* p) {
  float4 a = *reinterpret_cast<const float4*>(p);
  return Vec4<float>{{a.x, a.y, a.z, a.w}};
}
__device__ __forceinline__ Vec4<double> ldv4(const double* p) {
  double2 a = *reinterpret_cast<const double2*>(p);
  double2 b = *(reinterpret_cast<const double2*>(p) + 1);
  return Vec4<double>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void stv4(float* p, const Vec4<float>& v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void stv4(double* p, const Vec4<double>& v) {
  *reinterpret_cast<double2*>(p) = make_double2(v.v[0], v.v[1]);
  *(reinterpret_cast<double2*>(p) + 1) = make_double2(v.v[2], v.v[3]);
}

// Bodies may set `static constexpr bool kVec4 = true` and provide
// elem4(i, acc) for four consecutive elements starting at a multiple of 4.
template <class B, class = void>
struct Vec4Flag : std::false_type {};
template <class B>
struct Vec4Flag<B, std::void_t<decltype(B::kVec4)>> : std::integral_constant<bool, B::kVec4> {};

// -------------------------------------------------------- elementwise
// Body interface (all __device__):
//   bool skip() const
//   void elem(int64_t i, Acc3<T>& a)   (grid-stride over [0, n))
//   static constexpr bool kReduce
//   void finish(const Acc3<T>& tot)
template <typename T, class Body>
__global__ void __launch_bounds__(kBlock) vec_kernel(int64_t n, T* partials,
                                                     unsigned int* counter, Body body) {
  if (body.skip()) return;
  Acc3<T> a{T(0), T(0), T(0)};
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  if constexpr (Vec4Flag<Body>::value) {
    // four consecutive elements per thread with 128-bit accesses, then the tail
    const int64_t n4 = n >> 2;
    for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n4; i += stride) body.elem4(i << 2, a);
    for (int64_t i = (n4 << 2) + (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) body.elem(i, a);
  } else {
    for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) body.elem(i, a);
  }
  if constexpr (Body::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) body.finish(tot);
  }
}

}  // namespace sx

namespace sx {

// FP32 epilogues may provide out_acc4(row0, w[4], out[4], acc): out() and
// acc() of four consecutive rows in row order, same arithmetic, with their
// vector loads issued together; y must then be 16-byte aligned.
template <class E, class = void>
struct EpiRows4 : std::false_type {};
template <class E>
struct EpiRows4<E, std::void_t<decltype(&E::out_acc4)>> : std::true_type {};

// Diagonal-layout SpMV.  The entries of row r sit at vals[d * ld + r] on the
// diagonals d whose bit is set in mask[r]; no column indices are read.  A
// thread owns VEC consecutive rows (4 in FP32, 2 in FP64): for every
// diagonal it reads the rows' values with one vector load and their x
// operands with one or two aligned vector loads (two when the diagonal's
// offset is not a multiple of VEC, then shifted in registers).  The
// diagonals ascend in offset, which is the storage order of the sorted CSR
// row, and each row's sum runs over its stored diagonals in that order
// (from zero, rounded products, or fused multiply-adds for FMA), so the
// result is that of the CSR kernels.  Rows near the ends of the matrix,
// where a vector load could leave [0, n), take a row-per-thread pass.
struct DiaOffs {
  int32_t off[16];
};

// x operands of VEC rows from the two aligned vectors a (columns c - s ..)
// and b (the next VEC columns), s = c mod VEC
template <typename T, int VEC>
__device__ __forceinline__ void dia_shift(const T (&a)[VEC], const T (&b)[VEC], int s, T (&o)[VEC]) {
#pragma unroll
  for (int j = 0; j < VEC; ++j) o[j] = a[j];
#pragma unroll
  for (int sh = 1; sh < VEC; ++sh)
    if (s == sh) {
#pragma unroll
      for (int j = 0; j < VEC; ++j) o[j] = j + sh < VEC ? a[j + sh] : b[j + sh - VEC];
    }
}

// Bands: runs of diagonals with consecutive offsets (at most three long;
// a 2D 9-point stencil is three bands of three).  A band's x operands lie in
// one window of three aligned vectors read once, instead of two vectors per
// diagonal.  Bit d of a band mask is set when diagonal d starts a band.
struct DiaBands {
  int count;
  int start[16];
  int len[16];
};
__host__ __device__ constexpr DiaBands dia_bands(unsigned bands, int nd) {
  DiaBands t{0, {0}, {0}};
  for (int d = 0; d < nd; ++d) {
    if (d == 0 || ((bands >> d) & 1u)) {
      t.start[t.count] = d;
      t.len[t.count] = 1;
      ++t.count;
    } else {
      ++t.len[t.count - 1];
    }
  }
  return t;
}
// the band mask of sorted offsets (runs capped at three diagonals)
inline unsigned dia_band_mask(const int32_t* off, int nd) {
  unsigned m = 0;
  int run = 0;
  for (int d = 0; d < nd; ++d) {
    if (d == 0 || off[d] != off[d - 1] + 1 || run == 3) {
      m |= 1u << d;
      run = 1;
    } else {
      ++run;
    }
  }
  return m;
}
// x operands of VEC rows at window position q (the window: w[0], w[1], w[2]
// back to back), 0 <= q <= VEC + 1.  For four FP32 rows the window goes
// through three float4 values first: this exact form compiled to a much
// faster schedule than the same selection written over the arrays (10.6 vs
// 12.3 us back to back on the 1024^2 Q1 matrix).
__device__ __forceinline__ void win_shift4(const float4& a, const float4& b, const float4& c, int q, float (&o)[4]) {
  const float t[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
#pragma unroll
  for (int sh = 0; sh < 6; ++sh)
    if (q == sh) {
      o[0] = t[sh];
      o[1] = t[sh + 1];
      o[2] = t[sh + 2];
      o[3] = t[sh + 3];
    }
}
template <typename T, int VEC>
__device__ __forceinline__ void win_shift(const T (&w)[3][VEC], int q, T (&o)[VEC]) {
  if constexpr (VEC == 4 && std::is_same<T, float>::value) {
    win_shift4(make_float4(w[0][0], w[0][1], w[0][2], w[0][3]), make_float4(w[1][0], w[1][1], w[1][2], w[1][3]),
               make_float4(w[2][0], w[2][1], w[2][2], w[2][3]), q, o);
  } else {
    T t[3 * VEC];
#pragma unroll
    for (int i = 0; i < 3 * VEC; ++i) t[i] = w[i / VEC][i % VEC];
#pragma unroll
    for (int sh = 0; sh <= VEC + 1; ++sh)
      if (q == sh) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) o[j] = t[sh + j];
      }
  }
}
// Inner row groups [glo, ghi) of the diagonal layout (VEC whole rows whose
// aligned x vectors, two per diagonal or a three-vector window per band of
// up to three, all lie inside [0, n)) and the count of the other rows
__host__ __device__ inline void dia_ranges(int n, int omin, int omax, int vec, int& glo, int& ghi, int& nb) {
  const int groups = (n + vec - 1) / vec;
  const int need = vec - omin;
  glo = need <= 0 ? 0 : (need + vec - 1) / vec;
  const int lim = (n - omax - 2 * vec - 2) < (n - vec) ? (n - omax - 2 * vec - 2) : (n - vec);
  ghi = lim < 0 ? 0 : lim / vec + 1;
  glo = glo < groups ? glo : groups;
  ghi = ghi < groups ? ghi : groups;
  ghi = ghi > glo ? ghi : glo;
  const int head = glo * vec < n ? glo * vec : n;
  nb = head + (n - ghi * vec > 0 ? n - ghi * vec : 0);
}
// Epilogues that declare kBanded get the band kernels (the plain product and
// the solvers' hot epilogues); the others keep one window per diagonal,
// which bounds the number of kernel instantiations
template <class E, class = void>
struct EpiBanded : std::false_type {};
template <class E>
struct EpiBanded<E, std::void_t<decltype(E::kBanded)>> : std::integral_constant<bool, E::kBanded> {};

// Diagonals per batch of loads: every load of a batch is issued before the
// first product, with no condition on them (batch slots past the last
// diagonal re-read it and are masked off), so a thread waits for memory
// once per batch rather than once per diagonal.  (All nine diagonals of a
// 2D stencil in one batch measured no faster on the 1024^2 Q1 matrix and
// slower on the 3D ones: 104-206 registers per thread in the fused solver
// kernels instead of 64-80.)
constexpr int kDiaBatch = 4;
// the diagonal kernel for any count up to 16 (runtime count); smaller ND
// instantiations are for exactly ND diagonals
constexpr int kDiaGeneric = 16;

// Resident blocks asked of the compiler: three for the exact-count FP32
// kernels (at most 80 registers, every load of the vector path still in
// flight), two otherwise (the generic and FP64 kernels would spill).
// With bands (a third of the x registers) the FP32 kernels fit four blocks.
template <typename T, int ND, unsigned BANDS>
constexpr int dia_min_blocks() {
  return sizeof(T) == 4 && ND < 16 ? (BANDS != 0 && BANDS != (1u << ND) - 1 ? 4 : 3) : 2;
}

// Programmatic dependent launch: a kernel launched with it may start while
// the previous kernel in the stream finishes.  It lets its own dependents
// start at once (pdl_launch_dependents) and waits for the previous kernel's
// completion and memory (pdl_wait) before reading anything that kernel, or
// any before it, wrote.  Both are no-ops for a launch without it.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// One inner row group of the diagonal-layout SpMV (the kernel below).  PRE:
// the group's mask and values (never written by a kernel) are loaded before
// the wait for the previous kernel, and the epilogue's skip test after it;
// returns false when the launch is skipped.
template <typename T, int ND, class Epi, bool FMA, typename V, class Gather, unsigned BANDS, bool PRE = false>
__device__ __forceinline__ bool dia_group(int g, const V* __restrict__ vals, const uint16_t* __restrict__ mask,
                                          int64_t ld, DiaOffs offs, int ndr, const T* __restrict__ x,
                                          T* __restrict__ y, Epi epi, Gather gat, Acc3<T>& a) {
  constexpr int VEC = DiaVec<T>::kVec;
  constexpr bool kExact = ND < kDiaGeneric;
  constexpr int KB = kExact ? ND : kDiaBatch;
  const int r0 = g * VEC;
  T acc[VEC];
#pragma unroll
  for (int j = 0; j < VEC; ++j) acc[j] = T(0);
  unsigned m[VEC];  // one 8- or 4-byte load (r0 is a multiple of VEC)
  if constexpr (VEC == 4) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(mask + r0));
    m[0] = u.x & 0xFFFFu; m[1] = u.x >> 16; m[2] = u.y & 0xFFFFu; m[3] = u.y >> 16;
  } else {
    static_assert(VEC == 2, "DIA groups are 2 or 4 rows");
    const unsigned u = __ldg(reinterpret_cast<const unsigned*>(mask + r0));
    m[0] = u & 0xFFFFu; m[1] = u >> 16;
  }
  if constexpr (kExact) {
    // every diagonal's values of the group first (one vector each, the
    // loads that go to HBM); then band by band the x window (mostly L1/L2
    // hits) and the products in diagonal order
    constexpr unsigned kB = (BANDS != 0 && kExact) ? BANDS : (1u << (kExact ? ND : 1)) - 1;
    constexpr DiaBands kT = dia_bands(kB, kExact ? ND : 1);
    T v[ND][VEC];
#pragma unroll
    for (int d = 0; d < ND; ++d) vload(vals + (int64_t)d * ld + r0, v[d]);
    if constexpr (PRE) {
      pdl_wait();
      if (epi.skip()) return false;
    }
#pragma unroll
    for (int b = 0; b < kT.count; ++b) {
      // the band's x window: the vectors its last diagonal reaches, up to
      // window element (VEC - 1) + (L - 1) + (VEC - 1)
      const int d0 = kT.start[b], L = kT.len[b];
      const int nv = (L + 2 * VEC - 3) / VEC + 1;
      const int off = offs.off[d0];
      const int s = off & (VEC - 1);
      const int c = r0 + off - s;
      T w[3][VEC];
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (i < nv) gat.vec(x, c + i * VEC, w[i]);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k < L) {
          const int d = d0 + k;
          T xv[VEC];
          win_shift<T, VEC>(w, s + k, xv);
#pragma unroll
          for (int j = 0; j < VEC; ++j) {
            if ((m[j] >> d) & 1u) {
              if constexpr (FMA) acc[j] = fma(v[d][j], xv[j], acc[j]);
              else acc[j] = add_rn(acc[j], mul_rn(v[d][j], xv[j]));
            }
          }
        }
      }
    }
  } else {
    if constexpr (PRE) {
      pdl_wait();
      if (epi.skip()) return false;
    }
    // any count: batches of KB diagonals' value and x loads
#pragma unroll
    for (int d0 = 0; d0 < ND; d0 += KB) {
      if (d0 < ndr) {
        T v[KB][VEC], xa[KB][VEC], xb[KB][VEC];
#pragma unroll
        for (int t = 0; t < KB; ++t) {
          const int d = min(d0 + t, ndr - 1);
          vload(vals + (int64_t)d * ld + r0, v[t]);
          const int c = r0 + offs.off[d] - (offs.off[d] & (VEC - 1));
          gat.vec(x, c, xa[t]);
          gat.vec(x, c + VEC, xb[t]);
        }
#pragma unroll
        for (int t = 0; t < KB; ++t) {
          const int d = d0 + t;
          T xv[VEC];
          dia_shift<T, VEC>(xa[t], xb[t], offs.off[min(d, ndr - 1)] & (VEC - 1), xv);
#pragma unroll
          for (int j = 0; j < VEC; ++j) {
            if (d < ndr && ((m[j] >> d) & 1u)) {
              if constexpr (FMA) acc[j] = fma(v[t][j], xv[j], acc[j]);
              else acc[j] = add_rn(acc[j], mul_rn(v[t][j], xv[j]));
            }
          }
        }
      }
    }
  }
  // the group's VEC results with one 16-byte store, after the epilogue's
  // own loads and reduction terms (acc() takes the stored value as an
  // argument, never from y): loads placed after the store would wait
  // for it, as they may alias y (1.5x slower FP64 CG on the 1024^2 Q1
  // matrix).  Epilogues with a four-row form issue their vector loads
  // together.
  T o[VEC];
  if constexpr (EpiRows4<Epi>::value && VEC == 4) {
    epi.out_acc4(r0, acc, o, a);
  } else {
#pragma unroll
    for (int j = 0; j < VEC; ++j) o[j] = epi.out(r0 + j, acc[j]);
#pragma unroll
    for (int j = 0; j < VEC; ++j) epi.acc(r0 + j, o[j], a);
  }
  if constexpr (VEC == 4) *reinterpret_cast<float4*>(y + r0) = make_float4(o[0], o[1], o[2], o[3]);
  else *reinterpret_cast<double2*>(y + r0) = make_double2(o[0], o[1]);
  return true;
}

// One row outside the inner groups: every value and x element of the row
// loaded first (x at clamped, always valid columns; absent entries are
// masked off), then the storage-order sum.
template <typename T, int ND, class Epi, bool FMA, typename V, class Gather>
__device__ __forceinline__ void dia_row(int row, int n, const V* __restrict__ vals, const uint16_t* __restrict__ mask,
                                        int64_t ld, DiaOffs offs, int ndr, const T* __restrict__ x,
                                        T* __restrict__ y, Epi epi, Gather gat, Acc3<T>& a) {
  constexpr bool kExact = ND < kDiaGeneric;
  const unsigned mr = __ldg(mask + row);
  constexpr int RB = kExact ? ND : 8;  // diagonals per batch of loads
  T acc = T(0);
#pragma unroll
  for (int d0 = 0; d0 < ND; d0 += RB) {
    if (d0 < ndr) {
      T v[RB], xv[RB];
#pragma unroll
      for (int t2 = 0; t2 < RB; ++t2) {
        const int dd = min(d0 + t2, ndr - 1);
        v[t2] = (T)to_val(vals[(int64_t)dd * ld + row]);
        xv[t2] = gat(x, min(max(row + offs.off[dd], 0), n - 1));
      }
#pragma unroll
      for (int t2 = 0; t2 < RB; ++t2) {
        const int d = d0 + t2;
        if (d < ndr && ((mr >> d) & 1u)) {
          if constexpr (FMA) acc = fma(v[t2], xv[t2], acc);
          else acc = add_rn(acc, mul_rn(v[t2], xv[t2]));
        }
      }
    }
  }
  const T val = epi.out(row, acc);
  epi.acc(row, val, a);
  y[row] = val;
}

// BANDS: the band mask of an exact-count kernel (0: one band per diagonal).
// FULL: the grid has a thread for every inner group and every other row
// (each thread does one of them, straight-line code); else a grid-stride
// loop over the inner groups, then over the other rows.
template <typename T, int ND, class Epi, bool FMA = false, typename V = T, class Gather = GatherPlain<T>,
          unsigned BANDS = 0, bool FULL = false>
//
// (nd follows nrows: placed between offs and x, it measured 12.3 instead of
// 10.7 us back to back on the 1024^2 Q1 matrix with identical code, the
// parameters' offsets being the only difference)
__global__ void __launch_bounds__(kBlock, dia_min_blocks<T, ND, BANDS>()) spmv_dia_kernel(const V* __restrict__ vals,
                                                          const uint16_t* __restrict__ mask, int64_t ld,
                                                          DiaOffs offs, const T* __restrict__ x,
                                                          T* __restrict__ y, int64_t nrows, int nd, T* partials,
                                                          unsigned int* counter, Epi epi, Gather gat = Gather{}) {
  pdl_launch_dependents();
  constexpr int VEC = DiaVec<T>::kVec;
  // ND < kDiaGeneric: exactly ND diagonals, every loop straight-line code
  // (runtime bounds there split the unrolled loops into branches, and the
  // compiler then no longer issues later diagonals' x loads early: 1.45x
  // slower on the 1024^2 Q1 matrix); ND == kDiaGeneric: nd <= ND at runtime
  constexpr bool kExact = ND < kDiaGeneric;
  const int ndr = kExact ? ND : nd;
  Acc3<T> a{T(0), T(0), T(0)};
  const int n = (int)nrows;
  const int stride = (int)gridDim.x * kBlock;
  const int tid = (int)blockIdx.x * kBlock + (int)threadIdx.x;
  // inner groups take the vector path; the few rows outside them (near both
  // ends) take the row path, kept apart so that its code does not raise the
  // vector path's register count (a group-level branch between the two cost
  // 40 registers per thread and a third of the resident warps)
  int glo, ghi, nb;
  dia_ranges(n, offs.off[0], offs.off[ndr - 1], VEC, glo, ghi, nb);
  const int head = min(glo * VEC, n);
  const int span = ghi - glo;
  // every thread waits for the previous kernel (under a programmatic launch)
  // and tests the epilogue's skip after the wait, all alike; the inner groups
  // of a full grid load their values first
  if constexpr (FULL) {
    // the other rows first: their blocks are scheduled first and overlap
    // the inner groups, instead of lengthening the kernel's tail
    if (tid >= nb && tid - nb < span) {
      if (!dia_group<T, ND, Epi, FMA, V, Gather, BANDS, true>(glo + tid - nb, vals, mask, ld, offs, ndr, x, y, epi,
                                                              gat, a))
        return;
    } else {
      pdl_wait();
      if (epi.skip()) return;
      if (tid < nb)
        dia_row<T, ND, Epi, FMA, V, Gather>(tid < head ? tid : ghi * VEC + (tid - head), n, vals, mask, ld, offs,
                                            ndr, x, y, epi, gat, a);
    }
  } else {
    pdl_wait();
    if (epi.skip()) return;
    for (int g = glo + tid; g < ghi; g += stride)
      dia_group<T, ND, Epi, FMA, V, Gather, BANDS>(g, vals, mask, ld, offs, ndr, x, y, epi, gat, a);
    // the other rows go to the threads counted from the end of the grid,
    // which the grid-stride loop gave the fewest groups
    for (int t = stride - 1 - tid; t < nb; t += stride)
      dia_row<T, ND, Epi, FMA, V, Gather>(t < head ? t : ghi * VEC + (t - head), n, vals, mask, ld, offs, ndr, x, y,
                                          epi, gat, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

// Short-row SpMV: one thread per row, the row's K-entry window entirely in
// registers (no shared memory, no block barrier).  Every column/value load
// and then every gather of a row is issued before the first is used; the
// products and the sum then follow storage order (csr.rs:479-497), so the
// results are those of the other kernels.  Rows longer than K take a
// sequential tail loop.  Consecutive threads own consecutive rows, so a
// warp's k-th loads fall in a few consecutive lines that L1 serves to the
// following loads.
template <typename T, int K, class Epi, bool FMA = false, typename V = T, class Gather = GatherPlain<T>>
__global__ void __launch_bounds__(kBlock) spmv_short_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, const V* __restrict__ vals,
    const T* __restrict__ x, T* __restrict__ y, int64_t nrows, T* partials, unsigned int* counter, Epi epi,
    Gather gat = Gather{}) {
  if (epi.skip()) return;
  Acc3<T> a{T(0), T(0), T(0)};
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  for (int64_t row = (int64_t)blockIdx.x * kBlock + threadIdx.x; row < nrows; row += stride) {
    const int32_t s = __ldg(indptr + row), e = __ldg(indptr + row + 1);
    const int len = e - s;
    int col[K];
    T val[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool in = j < len;
      col[j] = in ? __ldg(indices + s + j) : 0;
      val[j] = in ? (T)to_val(vals[s + j]) : T(0);
    }
    T xv[K];
#pragma unroll
    for (int j = 0; j < K; ++j) xv[j] = j < len ? gat(x, col[j]) : T(0);
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j < len) {
        if constexpr (FMA) acc = fma(val[j], xv[j], acc);
        else acc = add_rn(acc, mul_rn(val[j], xv[j]));
      }
    }
    for (int32_t k = s + K; k < e; ++k) {  // rows longer than K
      const T vk = (T)to_val(vals[k]), xk = gat(x, __ldg(indices + k));
      if constexpr (FMA) acc = fma(vk, xk, acc);
      else acc = add_rn(acc, mul_rn(vk, xk));
    }
    const T v = epi.out(row, acc);
    y[row] = v;
    epi.acc(row, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

}  // namespace sx
