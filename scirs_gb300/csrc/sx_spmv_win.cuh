// Warp-streamed CSR SpMV, exact per-row summation order.
//
// Work decomposition.  The nonzeros are cut into units of kUnit = 256
// entries.  Every warp of the grid owns a contiguous run of units and walks
// it in windows of CAP entries (CAP / kUnit units), each window one stage of
// a per-warp ring of S shared-memory stages:
//   stage = [values: CAP x T][column indices: CAP x int32][row pointers: IPC x int32]
// The lanes fill a stage with 16-byte asynchronous copies (`cp.async.cg`,
// one commit group per window) of the values, the columns and the
// row-pointer slice of the rows the window touches, S - 1 windows ahead of
// the one being consumed.  A window is consumed in two passes:
//   pass 1  p_k = a_k * x[col_k] (rounded like the reference) into a per-warp
//           buffer; every gather of a lane is issued before the first is used
//           (PIPE: the gathers of window i + 1 are issued before window i is
//           summed);
//   pass 2  one lane per row sums its products in storage order.
// A row that runs past the end of a window keeps its partial sum in a
// register and continues in the next window of the same warp, so every row
// is summed strictly left to right from 0 -- the order of csr.rs:479-497
// and csr_array.rs:569-593 -- whatever the window boundaries.
//
// Row ownership.  tile_row[u] is the first row r with indptr[r+1] > u*kUnit
// (tile_row[0] = 0, tile_row[units] = nrows).  A window [W0, W1) serves rows
// tile_row[W0/kUnit] .. tile_row[W1/kUnit]; the last of them may continue.  A
// warp skips rows that started before its own first unit (the warp before
// finishes them) and, after its last unit, runs over into the following
// units until its own last row ends.  Empty rows are written by the window
// whose range holds their row pointer (ends included).
//
// Copies round their byte counts up to 16 and may read up to 15 bytes past
// the last element; every device array carries 64 bytes of slack for that.
#pragma once

#include <cstdint>

#include "sx_internal.h"
#include "sx_kernels.cuh"

namespace sx {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// 16-byte global -> shared copy, completion tracked per thread by commit groups
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename T, int CAP, int S, bool FMA>
struct WinCfg {
  static constexpr int kWarpsPerBlock = kBlock / 32;
  static constexpr int kUnits = CAP / kUnit;           // units per window
  static constexpr int kIpc = CAP / 4 + 8;             // row-pointer slots per stage
  static constexpr int kStage = CAP * (int)sizeof(T) + CAP * 4 + kIpc * 4;
  // the ring, then the products (exact) or the gathered x (FMA)
  static constexpr int kWarpBytes = S * kStage + CAP * (int)sizeof(T);
  static constexpr int kSmem = kWarpsPerBlock * kWarpBytes;
  static_assert(CAP % kUnit == 0, "CAP must be a multiple of kUnit");
  static_assert(kIpc % 4 == 0, "row-pointer slice must stay 16-byte aligned");
};

// window header, written by lane 0 when the window's copies are issued
struct WinHdr {
  int32_t w0, w1;   // nonzero range [w0, w1)
  int32_t rs, re;   // first row, row that may continue (nrows if none)
  int32_t a0;       // first row pointer index held in the stage; -1: read indptr
  int32_t runover;  // 1: only row rs, continuing from the carry; re = its end pointer
  int32_t pad0, pad1;
};

template <typename T, int CAP, int S, class Epi, bool FMA, bool PIPE>
__global__ void __launch_bounds__(kBlock) spmv_win_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, const T* __restrict__ vals,
    const int32_t* __restrict__ tile_row, const T* __restrict__ x, T* __restrict__ y, int64_t nrows,
    int64_t nnz, int64_t units, T* partials, unsigned int* counter, Epi epi) {
  using C = WinCfg<T, CAP, S, FMA>;
  if (epi.skip()) return;
  extern __shared__ __align__(128) unsigned char win_smem[];
  __shared__ WinHdr hdrs[C::kWarpsPerBlock][S];

  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* wbase = win_smem + (size_t)wib * C::kWarpBytes;
  WinHdr* hdr = hdrs[wib];
  T* xs = reinterpret_cast<T*>(wbase + S * C::kStage);  // products, or x for FMA

  const int64_t nw = (int64_t)gridDim.x * C::kWarpsPerBlock;
  const int64_t gw = (int64_t)blockIdx.x * C::kWarpsPerBlock + wib;
  const int64_t ub = gw * units / nw, ue = (gw + 1) * units / nw;
  const int64_t own0 = ub * kUnit;
  const int64_t nmain = (ue - ub + C::kUnits - 1) / C::kUnits;

  Acc3<T> acc3{T(0), T(0), T(0)};

  // tile_row at window boundaries, 31 windows per batch (lane l: boundary 31b + l)
  auto load_batch = [&](int64_t b) -> int32_t {
    const int64_t k = 31 * b + lane;
    return k <= nmain ? __ldg(tile_row + ub + min(k * C::kUnits, ue - ub)) : 0;
  };
  int64_t bp = 0;
  int32_t trp = nmain > 0 ? load_batch(0) : 0;
  int32_t trn = nmain > 31 ? load_batch(1) : 0;

  // run-over: the row that continues past this warp's last unit, if it started here
  int64_t ustop = ue;
  int32_t pr = -1, pr_end = 0;

  // fills stage i % S with window i (warp-uniform call; every lane copies)
  auto produce = [&](int64_t i) {
    WinHdr h;
    int64_t w0, w1;
    if (i < nmain) {
      const int64_t b = i / 31;
      if (b > bp) {  // advance to the next batch and prefetch the one after
        trp = trn;
        bp = b;
        if (31 * (b + 1) <= nmain) trn = load_batch(b + 1);
      }
      const int j = (int)(i - 31 * b);
      const int64_t u0 = ub + i * C::kUnits;
      const int64_t u1 = min(u0 + C::kUnits, ue);
      w0 = u0 * kUnit;
      w1 = min(u1 * kUnit, nnz);
      h.rs = __shfl_sync(0xffffffffu, trp, j);
      h.re = __shfl_sync(0xffffffffu, trp, j + 1);
      h.runover = 0;
      const int32_t last = min((int64_t)h.re, nrows - 1) + 1;  // highest pointer index needed
      const int32_t a0 = h.rs & ~3;
      const int32_t a1 = (last + 1 + 3) & ~3;
      h.a0 = (a1 - a0 <= C::kIpc) ? a0 : -1;
    } else {
      const int64_t u0 = ue + (i - nmain) * C::kUnits;
      const int64_t u1 = min(u0 + C::kUnits, ustop);
      w0 = u0 * kUnit;
      w1 = min(u1 * kUnit, (int64_t)pr_end);
      h.rs = pr;
      h.re = pr_end;
      h.runover = 1;
      h.a0 = -1;
    }
    h.w0 = (int32_t)w0;
    h.w1 = (int32_t)w1;
    const int s = (int)(i % S);
    unsigned char* st = wbase + (size_t)s * C::kStage;
    if (lane == 0) hdr[s] = h;
    const int64_t cnt = w1 - w0;
    const int nv = (int)((cnt * (int64_t)sizeof(T) + 15) >> 4);
    const int nc = (int)((cnt * 4 + 15) >> 4);
    int ni = 0;
    if (h.a0 >= 0) {
      const int32_t last = min((int64_t)h.re, nrows - 1) + 1;
      ni = (((last + 1 + 3) & ~3) - h.a0) >> 2;
    }
    const char* gv = reinterpret_cast<const char*>(vals + w0);
    const char* gc = reinterpret_cast<const char*>(indices + w0);
    const char* gp = reinterpret_cast<const char*>(indptr + (h.a0 >= 0 ? h.a0 : 0));
    for (int j = lane; j < nv; j += 32) cp_async16(st + 16 * j, gv + 16 * j);
    for (int j = lane; j < nc; j += 32) cp_async16(st + CAP * sizeof(T) + 16 * j, gc + 16 * j);
    for (int j = lane; j < ni; j += 32) cp_async16(st + CAP * (sizeof(T) + 4) + 16 * j, gp + 16 * j);
  };

  // one commit group per ring slot, empty ones included, so that window i
  // is always group i and the waits below count groups uniformly
  const int64_t first = min((int64_t)S, nmain);
  for (int64_t i = 0; i < first; ++i) { produce(i); cp_async_commit(); }
  if (ue > ub && ue < units) {
    const int32_t p = __ldg(tile_row + ue);
    if (p < nrows) {
      const int32_t ps = __ldg(indptr + p), pe = __ldg(indptr + p + 1);
      if (ps >= own0 && (int64_t)ps < ue * kUnit) {
        pr = p;
        pr_end = pe;
        ustop = ((int64_t)pe - 1) / kUnit + 1;
      }
    }
  }
  const int64_t nwin = nmain + (ustop - ue + C::kUnits - 1) / C::kUnits;
  for (int64_t i = first; i < S; ++i) {
    if (i < nwin) produce(i);
    cp_async_commit();
  }

  T carry = T(0);
  constexpr int PER = CAP / 32;
  T xv[PER];
  // pass 1a: issue every x gather of this lane for the window in stage s
  auto gather = [&](int s, int cnt) {
    const int32_t* sc = reinterpret_cast<const int32_t*>(wbase + (size_t)s * C::kStage + CAP * sizeof(T));
    int col[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) col[j] = (lane + 32 * j < cnt) ? sc[lane + 32 * j] : -1;
#pragma unroll
    for (int j = 0; j < PER; ++j) xv[j] = col[j] >= 0 ? __ldg(x + col[j]) : T(0);
  };
  // pass 1b: products (exact) or gathered x (FMA) into the warp's buffer
  auto apply = [&](int s, int cnt) {
    const T* sv = reinterpret_cast<const T*>(wbase + (size_t)s * C::kStage);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int k = lane + 32 * j;
      if (k < cnt) xs[k] = FMA ? xv[j] : mul_rn(sv[k], xv[j]);
    }
  };
  // pass 2: one lane per row, storage order
  auto sums = [&](const WinHdr& h, int s) {
    const unsigned char* st = wbase + (size_t)s * C::kStage;
    const T* sv = reinterpret_cast<const T*>(st);
    const int32_t* sp = reinterpret_cast<const int32_t*>(st + CAP * (sizeof(T) + 4));
    const int cnt = h.w1 - h.w0;
    if (h.runover) {
      if (lane == 0) {
        T acc = carry;
        for (int k = 0; k < cnt; ++k) {
          if constexpr (FMA) acc = fma(sv[k], xs[k], acc);
          else acc = add_rn(acc, xs[k]);
        }
        if (h.re <= h.w1) {
          const T v = epi.out(h.rs, acc);
          y[h.rs] = v;
          epi.acc(h.rs, v, acc3);
        }
        carry = acc;
      }
      carry = __shfl_sync(0xffffffffu, carry, 0);
    } else {
      const int32_t rlast = (int32_t)min((int64_t)h.re, nrows - 1);
      T mycarry = T(0);
      for (int32_t r = h.rs + lane; r <= rlast; r += 32) {
        int32_t ipr, ipe;
        if (h.a0 >= 0) { ipr = sp[r - h.a0]; ipe = sp[r + 1 - h.a0]; }
        else { ipr = __ldg(indptr + r); ipe = __ldg(indptr + r + 1); }
        if ((int64_t)ipr < own0) continue;  // started in the previous warp's units
        const int32_t beg = max(ipr, h.w0), end = min(ipe, h.w1);
        T acc = ipr < h.w0 ? carry : T(0);
        for (int32_t k = beg - h.w0; k < end - h.w0; ++k) {
          if constexpr (FMA) acc = fma(sv[k], xs[k], acc);
          else acc = add_rn(acc, xs[k]);
        }
        if (ipe <= h.w1) {
          const T v = epi.out(r, acc);
          y[r] = v;
          epi.acc(r, v, acc3);
        } else {
          mycarry = acc;
        }
      }
      if (h.re < nrows) carry = __shfl_sync(0xffffffffu, mycarry, (h.re - h.rs) & 31);
    }
  };
  // refill the consumed stage S windows ahead (an empty group past the end)
  auto release = [&](int64_t i) {
    __syncwarp();
    if (i + S < nwin) produce(i + S);
    cp_async_commit();
  };
  if constexpr (!PIPE) {
    for (int64_t i = 0; i < nwin; ++i) {
      const int s = (int)(i % S);
      cp_async_wait<S - 1>();  // window i is group i; S - 1 younger groups may be pending
      __syncwarp();
      const WinHdr h = hdr[s];
      gather(s, h.w1 - h.w0);
      apply(s, h.w1 - h.w0);
      __syncwarp();
      sums(h, s);
      release(i);
    }
  } else {
    // the gathers of window i + 1 are in flight while window i is summed
    static_assert(!PIPE || S >= 2, "pipelined gathers need two stages");
    WinHdr h{};
    if (nwin > 0) {
      cp_async_wait<S - 1>();
      __syncwarp();
      h = hdr[0];
      gather(0, h.w1 - h.w0);
    }
    for (int64_t i = 0; i < nwin; ++i) {
      const int s = (int)(i % S);
      apply(s, h.w1 - h.w0);
      __syncwarp();
      WinHdr hn{};
      if (i + 1 < nwin) {
        const int sn = (int)((i + 1) % S);
        cp_async_wait<S - 2>();  // window i + 1 is group i + 1
        __syncwarp();
        hn = hdr[sn];
        gather(sn, hn.w1 - hn.w0);
      }
      sums(h, s);
      release(i);
      h = hn;
    }
  }
  cp_async_wait<0>();
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(acc3, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

}  // namespace sx

