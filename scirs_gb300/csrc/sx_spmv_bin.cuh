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
//  - long groups (the first bin_long_groups groups, rows up to thousands
//    of entries): one thread block per group.  Round by round, its 256
//    threads load 256 consecutive entries of every row of the group with
//    coalesced loads, form the rounded products and stage them in shared
//    memory; then lane r of warp 0 adds row r's products in storage order.
//    A row's entries are thus loaded by the whole block while its sum stays
//    sequential.
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
  T prod[32][kBlock + 1];  // [row of the group][entry of the round], padded
  int32_t start[32], len[32];
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
        // ---- exact: one long group of 32 rows per block.  A round covers
        // 256 consecutive entries of every row: thread t forms the product
        // at position c0 + t of each row (loads coalesced across threads,
        // 16 rows' loads in flight), staged in shared memory; lane r of
        // warp 0 then adds row r's products of the round in storage order.
        int32_t row = -1;
        if (w == 0) {
          const int64_t pidx = it * 32 + lane;
          row = pidx < nrows ? __ldg(perm + pidx) : -1;
          const int32_t s0 = row >= 0 ? __ldg(indptr + row) : 0;
          sm.start[lane] = s0;
          sm.len[lane] = row >= 0 ? __ldg(indptr + row + 1) - s0 : 0;
        }
        __syncthreads();
        int32_t lmax = 0;
#pragma unroll 8
        for (int r = 0; r < 32; ++r) lmax = max(lmax, sm.len[r]);
        T acc = T(0);
        for (int32_t c0 = 0; c0 < lmax; c0 += kBlock) {
          const int32_t j = c0 + (int32_t)threadIdx.x;
#pragma unroll
          for (int h = 0; h < 32; h += 16) {
            int32_t col[16];
            T v[16];
            // unconditional loads at clamped, always valid positions (so
            // the 16 rows' loads issue back to back); positions past a
            // row's end are masked when summed, not here
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int32_t lq = sm.len[h + q];
              const int32_t k = lq > 0 ? sm.start[h + q] + min(j, lq - 1) : 0;
              col[q] = __ldg(indices + k);
              v[q] = __ldg(vals + k);
            }
#pragma unroll
            for (int q = 0; q < 16; ++q) sm.prod[h + q][threadIdx.x] = mul_rn(v[q], __ldg(x + col[q]));
          }
          __syncthreads();
          if (w == 0) {
            const int32_t cnt = min(kBlock, sm.len[lane] - c0);
            const T* pr = sm.prod[lane];
            int32_t q = 0;
            for (; q + 8 <= cnt; q += 8) {
#pragma unroll
              for (int u = 0; u < 8; ++u) acc = add_rn(acc, pr[q + u]);
            }
            for (; q < cnt; ++q) acc = add_rn(acc, pr[q]);
          }
          __syncthreads();
        }
        if (w == 0 && row >= 0) {
          const T v = epi.out(row, acc);
          y[row] = v;
          epi.acc(row, v, a);
        }
        __syncthreads();  // start/len are rewritten by the next group
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
