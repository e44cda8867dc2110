// Sliced SpMV for matrices with long rows (power-law row lengths).
//
// Layout (built once per matrix, beside the CSR arrays): the rows ordered by
// length, longest first (bin_perm, a stable counting sort), cut into slices
// of 32 rows.  Slice s stores position j of its row q at sl_base[s] + 32 j + q
// (columns and values), zero-padded to the slice's longest row, and
// sl_len[32 s + q] is that row's length.  A warp reading position j of a
// slice reads 32 consecutive entries, so every matrix load is coalesced
// whatever the row lengths, and sorting keeps the padding small (0.1 % on a
// power-law matrix of 4M rows).  Only the x gathers stay random.
//
// Work items, longest first:
//  - big slices (longest row above kSlBig entries).  Exact mode: one block
//    per slice.  Warps 1-7 (producers) load the next kSlRound positions of
//    every row of the slice, gather x and stage the rounded products in one
//    of two shared-memory buffers; lane q of warp 0 (the consumer) adds row
//    q's products in storage order.  Named barriers hand the two buffers back
//    and forth, so the products of round k + 1 are formed while round k is
//    summed.  FMA mode: one warp per row of these slices instead
//    (lane-strided fused multiply-adds over the CSR arrays, then a fixed
//    shuffle tree), which keeps the long rows off a serial chain.
//  - mid slices: one warp per slice; lane q sums row q in registers, the
//    loads of kSlU positions in flight together.
//  - short slices (longest row at most kSlShort entries): kSlK slices per
//    warp, all their loads in flight together.
// Exact mode sums every row left to right from 0 with rounded products (the
// order of csr.rs:479-497 and csr_array.rs:569-593), bit-identical to the CSR
// kernels.  FMA mode (solver-internal FP64) fuses the products: a few ulp per
// row, deterministic run to run.
#pragma once

#include "sx_kernels.cuh"

namespace sx {

constexpr int kSlProd = kWarps - 1;          // producer warps of a big slice
constexpr int kSlPer = 8;                    // positions per producer lane and round
constexpr int kSlRound = kSlProd * kSlPer;   // positions per round of a big slice
constexpr int kSlU = 8;                      // positions per batch of a mid slice
constexpr int kSlK = 4;                      // short slices per warp

template <typename T>
struct SlSmem {
  T prod[2][kSlRound][32];  // [buffer][position of the round][row of the slice]
};

// Named barriers 1-4 (0 is __syncthreads): 1 + b "buffer b is full",
// 3 + b "buffer b is free"; every one counts all kBlock threads.
template <int ID>
__device__ __forceinline__ void bar_wait() {
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(kBlock) : "memory");
}
template <int ID>
__device__ __forceinline__ void bar_signal() {
  asm volatile("bar.arrive %0, %1;" ::"n"(ID), "n"(kBlock) : "memory");
}

// Work items of one launch: big-slice items (FMA: 8 rows per item), then the
// mid slices by 8, then the short slices by 8 * kSlK.
struct SlItems {
  int64_t big, mid, total;
  __host__ __device__ SlItems(int64_t nslices, int64_t nbig, int64_t nshort0, bool fma) {
    big = fma ? nbig * (32 / kWarps) : nbig;
    mid = (nshort0 - nbig + kWarps - 1) / kWarps;
    total = big + mid + (nslices - nshort0 + kWarps * kSlK - 1) / (kWarps * kSlK);
  }
};

template <typename T, class Epi, bool FMA>
__global__ void __launch_bounds__(kBlock, 3) spmv_sliced_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, const T* __restrict__ vals,
    const int32_t* __restrict__ perm, const int32_t* __restrict__ scols, const T* __restrict__ svals,
    const int64_t* __restrict__ sbase, const int32_t* __restrict__ slen, int64_t nrows, int64_t nslices,
    int64_t nbig, int64_t nshort0, const T* __restrict__ x, T* __restrict__ y, T* partials, unsigned int* counter,
    Epi epi) {
  extern __shared__ __align__(16) unsigned char sl_smem[];
  if (epi.skip()) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Acc3<T> a{T(0), T(0), T(0)};
  auto put = [&](int64_t row, T acc) {
    const T v = epi.out(row, acc);
    y[row] = v;
    epi.acc(row, v, a);
  };
  const SlItems items(nslices, nbig, nshort0, FMA);
  for (int64_t it = blockIdx.x; it < items.total; it += gridDim.x) {
    if (it < items.big) {
      if constexpr (FMA) {
        // ---- one long row per warp, lane-strided, then a shuffle tree
        const int64_t pidx = it * kWarps + w;
        if (pidx < nrows) {
          const int32_t row = __ldg(perm + pidx);
          const int32_t s = __ldg(indptr + row), e = __ldg(indptr + row + 1);
          T acc = T(0);
          int32_t k = s + lane;
          for (; k + 96 < e; k += 128) {
            const int32_t c0 = __ldg(indices + k), c1 = __ldg(indices + k + 32);
            const int32_t c2 = __ldg(indices + k + 64), c3 = __ldg(indices + k + 96);
            const T v0 = __ldg(vals + k), v1 = __ldg(vals + k + 32), v2 = __ldg(vals + k + 64),
                    v3 = __ldg(vals + k + 96);
            const T x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
            acc = fma(v0, x0, acc);
            acc = fma(v1, x1, acc);
            acc = fma(v2, x2, acc);
            acc = fma(v3, x3, acc);
          }
          for (; k < e; k += 32) acc = fma(__ldg(vals + k), __ldg(x + __ldg(indices + k)), acc);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) put(row, acc);
        }
      } else {
        // ---- exact: one big slice per block, producers and one consumer
        SlSmem<T>& sm = *reinterpret_cast<SlSmem<T>*>(sl_smem);
        const int64_t B = __ldg(sbase + it);
        const int32_t Lg = (int32_t)((__ldg(sbase + it + 1) - B) >> 5);
        const int R = (Lg + kSlRound - 1) / kSlRound;
        if (w == 0) {
          const int64_t p = it * 32 + lane;
          const int32_t len = __ldg(slen + p);
          T acc = T(0);
          for (int k = 0; k < R; ++k) {
            const int b = k & 1;
            if (b) bar_wait<2>();
            else bar_wait<1>();
            const int32_t cnt = min(kSlRound, len - k * kSlRound);
            const T* pr = &sm.prod[b][0][lane];
            int32_t q = 0;
            for (; q + 8 <= cnt; q += 8) {
#pragma unroll
              for (int u = 0; u < 8; ++u) acc = add_rn(acc, pr[(q + u) * 32]);
            }
            for (; q < cnt; ++q) acc = add_rn(acc, pr[q * 32]);
            if (b) bar_signal<4>();
            else bar_signal<3>();
          }
          if (p < nrows) put(__ldg(perm + p), acc);
        } else {
          const int pw = w - 1;
          for (int k = 0; k < R; ++k) {
            const int b = k & 1;
            if (k >= 2) {
              if (b) bar_wait<4>();
              else bar_wait<3>();
            }
            const int32_t c0 = k * kSlRound;
            int32_t c[kSlPer];
            T v[kSlPer];
            // positions past the slice's end load its last position again
            // (always valid); the consumer stops at each row's length
#pragma unroll
            for (int i = 0; i < kSlPer; ++i) {
              const int64_t o = B + (int64_t)min(c0 + pw + kSlProd * i, Lg - 1) * 32 + lane;
              c[i] = __ldcs(scols + o);
              v[i] = __ldcs(svals + o);
            }
#pragma unroll
            for (int i = 0; i < kSlPer; ++i) sm.prod[b][pw + kSlProd * i][lane] = mul_rn(v[i], __ldg(x + c[i]));
            if (b) bar_signal<2>();
            else bar_signal<1>();
          }
          // the consumer's release of the last one or two rounds, so that
          // every barrier is back at zero for the next slice
          for (int k = max(R - 2, 0); k < R; ++k) {
            if (k & 1) bar_wait<4>();
            else bar_wait<3>();
          }
        }
      }
    } else if (it < items.big + items.mid) {
      // ---- mid slice: one per warp, lane q sums row q in registers
      const int64_t g = nbig + (it - items.big) * kWarps + w;
      if (g < nshort0) {
        const int64_t B = __ldg(sbase + g);
        const int32_t Lg = (int32_t)((__ldg(sbase + g + 1) - B) >> 5);
        const int64_t p = g * 32 + lane;
        const int32_t len = __ldg(slen + p);
        T acc = T(0);
        for (int32_t j0 = 0; j0 < Lg; j0 += kSlU) {
          int32_t c[kSlU];
          T v[kSlU], xv[kSlU];
#pragma unroll
          for (int u = 0; u < kSlU; ++u) {
            const int64_t o = B + (int64_t)min(j0 + u, Lg - 1) * 32 + lane;
            c[u] = __ldcs(scols + o);
            v[u] = __ldcs(svals + o);
          }
#pragma unroll
          for (int u = 0; u < kSlU; ++u) xv[u] = __ldg(x + c[u]);
          // past the row's end the term is -0, which leaves every sum
          // unchanged (x + -0 = x in round-to-nearest, also for x = +-0)
#pragma unroll
          for (int u = 0; u < kSlU; ++u) {
            if constexpr (FMA) acc = j0 + u < len ? fma(v[u], xv[u], acc) : acc;
            else acc = add_rn(acc, j0 + u < len ? mul_rn(v[u], xv[u]) : T(-0.0));
          }
        }
        if (p < nrows) put(__ldg(perm + p), acc);
      }
    } else {
      // ---- kSlK short slices per warp, all their loads in flight together
      const int64_t g0 = nshort0 + ((it - items.big - items.mid) * kWarps + w) * kSlK;
      int64_t Bk[kSlK];
      int32_t Lk[kSlK], lenk[kSlK];
#pragma unroll
      for (int k = 0; k < kSlK; ++k) {
        const bool ok = g0 + k < nslices;
        Bk[k] = ok ? __ldg(sbase + g0 + k) : 0;
        Lk[k] = ok ? (int32_t)((__ldg(sbase + g0 + k + 1) - Bk[k]) >> 5) : 0;
        lenk[k] = ok ? __ldg(slen + (g0 + k) * 32 + lane) : 0;
      }
      int32_t c[kSlK][kSlShort];
      T v[kSlK][kSlShort], xv[kSlK][kSlShort];
#pragma unroll
      for (int k = 0; k < kSlK; ++k)
#pragma unroll
        for (int u = 0; u < kSlShort; ++u) {
          c[k][u] = u < Lk[k] ? __ldcs(scols + Bk[k] + u * 32 + lane) : 0;
          v[k][u] = u < Lk[k] ? __ldcs(svals + Bk[k] + u * 32 + lane) : T(0);
        }
#pragma unroll
      for (int k = 0; k < kSlK; ++k)
#pragma unroll
        for (int u = 0; u < kSlShort; ++u) xv[k][u] = u < Lk[k] ? __ldg(x + c[k][u]) : T(0);
#pragma unroll
      for (int k = 0; k < kSlK; ++k) {
        T acc = T(0);
#pragma unroll
        for (int u = 0; u < kSlShort; ++u) {
          if constexpr (FMA) acc = u < lenk[k] ? fma(v[k][u], xv[k][u], acc) : acc;
          else acc = add_rn(acc, u < lenk[k] ? mul_rn(v[k][u], xv[k][u]) : T(-0.0));
        }
        const int64_t p = (g0 + k) * 32 + lane;
        if (g0 + k < nslices && p < nrows) put(__ldg(perm + p), acc);
      }
    }
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

}  // namespace sx
