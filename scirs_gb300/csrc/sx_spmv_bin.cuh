// Length-binned SpMV for matrices with long rows (power-law row lengths).
//
// The rows are ordered by length, longest first (bin_perm, a stable counting
// sort built once per matrix), and handled in groups of 32 rows of similar
// length, so that the 32 lanes of a warp each sum one row at the same time:
// every FP64 instruction then has all its lanes busy.  That matters on
// GB300, whose FP64 pipe issues two lanes per clock per SM: an instruction
// with one active lane costs as much as a full warp (measured: a one-lane
// dependent DFMA chain takes ~65 clocks per step).
//
// Exact mode (the reference's order: sum = 0, then sum = sum + a*x in
// storage order, products rounded, csr.rs:479-497):
//  - long groups (the first bin_nlong_groups groups, rows up to thousands
//    of entries): one thread block per group.  Its 8 warps load eight
//    32-entry chunks of every row of the group with coalesced loads, form
//    the rounded products and stage them in shared memory; then lane r of
//    warp 0 adds row r's products in storage order.  A row's entries are
//    thus loaded by 8 warps in parallel while its sum stays sequential.
//  - short groups (rows of at most 32 entries): one warp per group, lane r
//    walks row r in storage order.
// FMA mode (solver-internal FP64, a few ulp per row): long rows get one
// warp each (lane-strided fused multiply-adds, then a fixed shuffle tree);
// short rows as above with fused multiply-adds.  The result is
// deterministic run to run in both modes.
#pragma once

#include "sx_kernels.cuh"

namespace sx {

template <typename T>
struct BinSmem {
  T prod[kWarps][32][33];  // [chunk][row of the group][entry of the chunk]
};

template <typename T, class Epi, bool FMA>
__global__ void __launch_bounds__(kBlock) spmv_bin_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, const T* __restrict__ vals,
    const int32_t* __restrict__ perm, int64_t nrows, int64_t nlong, int64_t sbeg, int64_t nitems,
    const T* __restrict__ x, T* __restrict__ y, T* partials, unsigned int* counter, Epi epi) {
  extern __shared__ __align__(16) unsigned char bin_smem[];
  if (epi.skip()) return;
  BinSmem<T>& sm = *reinterpret_cast<BinSmem<T>*>(bin_smem);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Acc3<T> a{T(0), T(0), T(0)};
  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    if (it < nlong) {
      if constexpr (!FMA) {
        // ---- exact: one long group of 32 rows per block
        const int64_t pidx = it * 32 + lane;
        const int32_t row = pidx < nrows ? __ldg(perm + pidx) : -1;
        const int32_t s = row >= 0 ? __ldg(indptr + row) : 0;
        const int32_t len = row >= 0 ? __ldg(indptr + row + 1) - s : 0;
        int32_t lmax = len;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        T acc = T(0);
        for (int32_t c0 = 0; c0 < lmax; c0 += kWarps * 32) {
          const int32_t cb = c0 + w * 32;
          if (cb < lmax) {
#pragma unroll 8
            for (int r = 0; r < 32; ++r) {
              const int32_t lr = __shfl_sync(0xffffffffu, len, r);
              const int32_t sr = __shfl_sync(0xffffffffu, s, r);
              if (cb < lr) {
                const int32_t j = cb + lane;
                T p = T(0);
                if (j < lr) {
                  const int32_t k = sr + j;
                  p = mul_rn(__ldg(vals + k), __ldg(x + __ldg(indices + k)));
                }
                sm.prod[w][r][lane] = p;
              }
            }
          }
          __syncthreads();
          if (w == 0) {
            // lane r: row r's products of this round, chunk by chunk in order
            for (int cw = 0; cw < kWarps; ++cw) {
              const int32_t cnt = min(32, len - (c0 + cw * 32));
              for (int32_t j = 0; j < cnt; ++j) acc = add_rn(acc, sm.prod[cw][lane][j]);
            }
          }
          __syncthreads();
        }
        if (w == 0 && row >= 0) {
          const T v = epi.out(row, acc);
          y[row] = v;
          epi.acc(row, v, a);
        }
      } else {
        // ---- FMA: one long row per warp, lane-strided, then a shuffle tree
        const int64_t pidx = it * kWarps + w;
        if (pidx < sbeg) {
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
          if (lane == 0) {
            const T v = epi.out(row, acc);
            y[row] = v;
            epi.acc(row, v, a);
          }
        }
      }
    } else {
      // ---- short rows: one group of 32 per warp, lane r walks row r
      const int64_t pidx = sbeg + ((it - nlong) * kWarps + w) * 32 + lane;
      if (pidx < nrows) {
        const int32_t row = __ldg(perm + pidx);
        const int32_t s = __ldg(indptr + row), e = __ldg(indptr + row + 1);
        T acc = T(0);
        int32_t k = s;
        for (; k + 3 < e; k += 4) {
          const int32_t c0 = __ldg(indices + k), c1 = __ldg(indices + k + 1);
          const int32_t c2 = __ldg(indices + k + 2), c3 = __ldg(indices + k + 3);
          const T v0 = __ldg(vals + k), v1 = __ldg(vals + k + 1), v2 = __ldg(vals + k + 2),
                  v3 = __ldg(vals + k + 3);
          const T x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
          if constexpr (FMA) {
            acc = fma(v0, x0, acc);
            acc = fma(v1, x1, acc);
            acc = fma(v2, x2, acc);
            acc = fma(v3, x3, acc);
          } else {
            acc = add_rn(acc, mul_rn(v0, x0));
            acc = add_rn(acc, mul_rn(v1, x1));
            acc = add_rn(acc, mul_rn(v2, x2));
            acc = add_rn(acc, mul_rn(v3, x3));
          }
        }
        for (; k < e; ++k) {
          const T vk = __ldg(vals + k), xk = __ldg(x + __ldg(indices + k));
          if constexpr (FMA) acc = fma(vk, xk, acc);
          else acc = add_rn(acc, mul_rn(vk, xk));
        }
        const T v = epi.out(row, acc);
        y[row] = v;
        epi.acc(row, v, a);
      }
    }
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

}  // namespace sx
