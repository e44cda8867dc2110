// Launch layer: y = op(x) with a compile-time epilogue for every operator
// kind of the library.  Included by the translation units that fuse solver
// scalar updates into operator applications.
#pragma once

#include <algorithm>
#include <type_traits>

#include "sx_internal.h"
#include "sx_kernels.cuh"
#include "sx_spmv_sliced.cuh"
#include "sx_spmv_win.cuh"

namespace sx {

// Epilogue that only stores A x.
template <typename T>
struct EpiPlain {
  static constexpr bool kBanded = true;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ T out(int64_t, T ax) const { return ax; }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// Epilogue y = b - A x (initial residuals: iterative.rs:78-79, :416-417, :677-678).
template <typename T>
struct EpiResid {
  const T* b;
  static constexpr bool kReduce = false;
  __device__ bool skip() const { return false; }
  __device__ T out(int64_t i, T ax) const { return sub_rn(b[i], ax); }
  __device__ void acc(int64_t, T, Acc3<T>&) const {}
  __device__ void finish(const Acc3<T>&) const {}
};

// Elementwise operators: identity, scaled identity, diagonal, Jacobi.  The
// product is rounded exactly as the reference's `x_i * d_i`
// (interface.rs:114, :160-163; preconditioners.rs:78-81).
template <typename T, class Epi>
__global__ void __launch_bounds__(kBlock) k_diag_apply(int64_t n, int kind, const T* __restrict__ d,
                                                       T scale, const T* __restrict__ x, T* y,
                                                       T* partials, unsigned int* counter, Epi epi) {
  if (epi.skip()) return;
  Acc3<T> a{T(0), T(0), T(0)};
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) {
    T ax;
    if (kind == SX_OP_ZERO) {
      ax = T(0);  // interface.rs:207: zeros whatever x holds
    } else {
      const T xi = x[i];
      ax = kind == SX_OP_IDENTITY ? xi : (kind == SX_OP_SCALED_IDENTITY ? mul_rn(xi, scale) : mul_rn(xi, d[i]));
    }
    T v = epi.out(i, ax);
    y[i] = v;
    epi.acc(i, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

// Epilogue over an already computed y (after a multi-kernel apply).
template <typename T, class Epi>
__global__ void __launch_bounds__(kBlock) k_epi_inplace(int64_t n, T* y, T* partials,
                                                        unsigned int* counter, Epi epi) {
  if (epi.skip()) return;
  Acc3<T> a{T(0), T(0), T(0)};
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) {
    T v = epi.out(i, y[i]);
    y[i] = v;
    epi.acc(i, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

// y = y + w elementwise (SumOperator: a + b, interface.rs:325-329), then the
// epilogue over y
template <typename T, class Epi>
__global__ void __launch_bounds__(kBlock) k_sum_epi(int64_t n, T* y, const T* __restrict__ w, T* partials,
                                                    unsigned int* counter, Epi epi) {
  if (epi.skip()) return;
  Acc3<T> a{T(0), T(0), T(0)};
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  for (int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += stride) {
    const T v = epi.out(i, add_rn(y[i], w[i]));
    y[i] = v;
    epi.acc(i, v, a);
  }
  if constexpr (Epi::kReduce) {
    Acc3<T> tot;
    if (grid_reduce3(a, partials, counter, tot) && threadIdx.x == 0) epi.finish(tot);
  }
}

constexpr int kSpmvItems = 8;

// Blocks of kBlock threads one SM holds at once for kernel Kern with `smem`
// bytes of dynamic shared memory, after opting Kern in to that much (queried
// once per kernel); -1 if it cannot run.  The cache is keyed by the kernel
// itself: every translation unit that instantiates a kernel template holds
// its own copy of the kernel, and the shared-memory opt-in belongs to that
// copy, so a cache shared by all units (keyed by template types) would leave
// the other units' copies without it.
template <auto Kern>
int resident_blocks_smem(int smem) {
  static int cached = 0;
  if (!cached) {
    int nb = 0;
    if ((smem > 48 * 1024 && cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                                 cudaSuccess) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, Kern, kBlock, smem) != cudaSuccess || nb < 1) {
      nb = -1;
      (void)cudaGetLastError();  // a refused query is a fallback, not an error of the next launch
    }
    cached = nb;
  }
  return cached;
}
// Blocks of kBlock threads one SM holds at once for kernel Kern (queried once).
template <auto Kern>
int resident_blocks() {
  const int nb = resident_blocks_smem<Kern>(0);
  return nb > 0 ? nb : 1;
}

// Window sizes, ring depths and gather pipelining of the windowed SpMV;
// SX_WIN_SHAPE selects the variant (0 default).
template <typename T, int V>
struct WinShape;
// (measured on the 4M-row power-law matrix: FP32 best without pipelining,
// FP64 best with three stages and pipelined gathers)
template <> struct WinShape<float, 0> { static constexpr int kCap = 256, kStages = 3; static constexpr bool kPipe = false; };
template <> struct WinShape<float, 1> { static constexpr int kCap = 256, kStages = 3; static constexpr bool kPipe = true; };
template <> struct WinShape<float, 2> { static constexpr int kCap = 256, kStages = 2; static constexpr bool kPipe = true; };
template <> struct WinShape<double, 0> { static constexpr int kCap = 256, kStages = 3; static constexpr bool kPipe = true; };
template <> struct WinShape<double, 1> { static constexpr int kCap = 256, kStages = 2; static constexpr bool kPipe = true; };
template <> struct WinShape<double, 2> { static constexpr int kCap = 256, kStages = 2; static constexpr bool kPipe = false; };

// Resident blocks per SM of one windowed SpMV variant (opts in to the
// dynamic shared memory once per instantiation); -1 if it cannot run.
template <typename T, int V, class Epi, bool FMA>
int win_resident_blocks() {
  using Sh = WinShape<T, V>;
  constexpr auto kern = spmv_win_kernel<T, Sh::kCap, Sh::kStages, Epi, FMA, Sh::kPipe>;
  return resident_blocks_smem<kern>(WinCfg<T, Sh::kCap, Sh::kStages, FMA>::kSmem);
}

template <typename T, int V, class Epi, bool FMA>
bool launch_win(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi, const ReduceArea& ra,
                int64_t blocks) {
  const int nb = win_resident_blocks<T, V, Epi, FMA>();
  if (nb <= 0) return false;
  using Sh = WinShape<T, V>;
  constexpr auto kern = spmv_win_kernel<T, Sh::kCap, Sh::kStages, Epi, FMA, Sh::kPipe>;
  constexpr int smem = WinCfg<T, Sh::kCap, Sh::kStages, FMA>::kSmem;
  // at least 4 units per warp, at most the resident blocks, at most the reduction area
  const int64_t by_units = (c.units + (kBlock / 32) * 4 - 1) / ((kBlock / 32) * 4);
  int64_t grid = std::min<int64_t>((int64_t)ctx->num_sms * nb, by_units);
  grid = std::max<int64_t>(1, std::min<int64_t>(grid, blocks));
  kern<<<(unsigned)grid, kBlock, smem, ctx->stream>>>(c.indptr, c.indices, (const T*)c.vals, c.tile_row, x, y,
                                                       c.nrows, c.nnz, c.units, (T*)ra.partials, ra.counter, epi);
  return true;
}

// Sliced SpMV launch (long-row matrices): big slices (exact) or their rows
// (FMA) first, then the mid and short slices; false when the matrix has no
// sliced layout or the kernel cannot be resident.
template <typename T, class Epi, bool FMA>
bool launch_sliced(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi, const ReduceArea& ra, int64_t blocks) {
  if (!ctx->bin || !c.sl_vals) return false;
  constexpr auto kern = spmv_sliced_kernel<T, Epi, FMA>;
  constexpr int smem = FMA ? 0 : (int)sizeof(SlSmem<T>);
  const int nb = resident_blocks_smem<kern>(smem);
  if (nb <= 0) return false;
  const SlItems items(c.sl_slices, c.sl_big, c.sl_short, FMA);
  int64_t grid = std::min<int64_t>((int64_t)ctx->num_sms * nb, items.total);
  grid = std::max<int64_t>(1, std::min<int64_t>(grid, blocks));
  kern<<<(unsigned)grid, kBlock, smem, ctx->stream>>>(c.indptr, c.indices, (const T*)c.vals, c.bin_perm, c.sl_cols,
                                                       (const T*)c.sl_vals, c.sl_base, c.sl_len, c.nrows, c.sl_slices,
                                                       c.sl_big, c.sl_short, x, y, (T*)ra.partials, ra.counter, epi);
  return true;
}

template <typename T, int ITEMS, class Epi, bool FMA, bool C16, int MINB, typename V = T>
void launch_pipe_minb(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi, const ReduceArea& ra,
                      int64_t blocks) {
  constexpr auto kern = spmv_pipe_kernel<T, ITEMS, Epi, FMA, C16, MINB, V>;
  const V* vals = std::is_same<V, T>::value ? (const V*)c.vals : (const V*)c.vals16;
  const int64_t grid = std::min<int64_t>(blocks, (int64_t)ctx->num_sms * resident_blocks<kern>());
  kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(c.indptr, c.indices, vals, x, y, c.nrows, blocks,
                                                    (T*)ra.partials, ra.counter, epi, c.col16, c.chunk_base,
                                                    GatherPlain<T>{});
}

// One diagonal-layout launch: as many blocks as the row groups need, at
// most the resident blocks of every SM (FULL: every group its own thread,
// the hardware handing out blocks as others finish).
template <auto Kern, bool FULL = false, typename T, typename V, class Epi, class Gather>
void dia_go(sx_ctx ctx, const DevCsr& c, const V* vals, const T* x, T* y, Epi epi, const ReduceArea& ra,
            Gather gat, const DiaOffs& offs, int64_t units) {
  int64_t grid = std::min<int64_t>((units + kBlock - 1) / kBlock, (int64_t)ctx->num_sms * resident_blocks<Kern>());
  if constexpr (FULL) {
    // a thread per inner group and per other row
    int glo = 0, ghi = 0, nb = 0;
    dia_ranges((int)c.nrows, c.dia_off[0], c.dia_off[c.dia_n - 1], DiaVec<T>::kVec, glo, ghi, nb);
    grid = std::max<int64_t>(1, ((int64_t)(ghi - glo) + nb + kBlock - 1) / kBlock);
  }
  if (ctx->pdl) {
    // programmatic dependent launch: the kernel may start while the previous
    // one in the stream finishes (it loads its matrix values meanwhile and
    // waits on the device before reading anything the previous one wrote):
    // 8.9 instead of 11.1 us per SpMV back to back on the 1024^2 Q1 matrix
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t le = cudaLaunchKernelEx(&cfg, Kern, vals, (const uint16_t*)c.dia_mask, (int64_t)c.dia_ld,
                                              offs, x, y, (int64_t)c.nrows, (int)c.dia_n, (T*)ra.partials,
                                              ra.counter, epi, gat);
    if (le == cudaSuccess) return;
    // a runtime that refuses the attribute: plain launches from here on (a
    // launch error proper comes back from the plain launch below)
    (void)cudaGetLastError();
    ctx->pdl = false;
  }
  Kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(vals, c.dia_mask, c.dia_ld, offs, x, y, c.nrows, c.dia_n,
                                                    (T*)ra.partials, ra.counter, epi, gat);
}

// Diagonal-layout SpMV launch (values of type V: T, or the FP16 copy);
// false when the matrix has no diagonal layout.
template <typename T, class Epi, bool FMA, typename V = T, class Gather = GatherPlain<T>>
bool launch_dia(sx_ctx ctx, const DevCsr& c, const V* vals, const T* x, T* y, Epi epi, const ReduceArea& ra,
                int64_t /*blocks*/, Gather gat = Gather{}) {
  if (!ctx->dia || !vals || c.dia_n <= 0 || !c.dia_mask) return false;
  // the layout's kernels read x and store y with 16-byte vectors: a caller's
  // vector at another alignment (a basis vector at an odd offset, say) takes
  // the CSR kernels instead
  if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0 || (reinterpret_cast<uintptr_t>(y) & 15u) != 0) return false;
  DiaOffs offs;
  for (int q = 0; q < 16; ++q) offs.off[q] = c.dia_off[q];
  const int64_t groups = (c.nrows + DiaVec<T>::kVec - 1) / DiaVec<T>::kVec;
  // band kernels for the stencil shapes here (2D Q1: three bands of three;
  // 3D 7-point: 1,1,3,1,1; 2D 5-point: 1,3,1; the learned factors of Q1: 3,2
  // and 2,3), for the plain product and the solvers' hot epilogues; FP32
  // ones on a full grid (four resident blocks: measured 10.4 vs 12.3 us
  // back to back on the 1024^2 Q1 matrix against a persistent grid)
  if constexpr (EpiBanded<Epi>::value) {
    if (ctx->dia_nd6 && ctx->dia_band) {
      constexpr bool kFull = sizeof(T) == 4;
      const unsigned bm = dia_band_mask(c.dia_off, c.dia_n);
      bool done = true;
      if (c.dia_n == 9 && bm == 0x49u)
        dia_go<spmv_dia_kernel<T, 9, Epi, FMA, V, Gather, 0x49u, kFull>, kFull>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
      else if (c.dia_n == 7 && bm == 0x67u)
        dia_go<spmv_dia_kernel<T, 7, Epi, FMA, V, Gather, 0x67u, kFull>, kFull>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
      else if (c.dia_n == 5 && bm == 0x13u)
        dia_go<spmv_dia_kernel<T, 5, Epi, FMA, V, Gather, 0x13u, kFull>, kFull>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
      else if (c.dia_n == 5 && bm == 0x09u)
        dia_go<spmv_dia_kernel<T, 5, Epi, FMA, V, Gather, 0x09u, kFull>, kFull>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
      else if (c.dia_n == 5 && bm == 0x05u)
        dia_go<spmv_dia_kernel<T, 5, Epi, FMA, V, Gather, 0x05u, kFull>, kFull>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
      else
        done = false;
      if (done) return true;
    }
  }
  // exact-count kernels for the stencils here (5: 2D 5-point and the learned
  // factors, 7: 3D 7-point, 9: 2D Q1), the generic one for any other count
  // (and for every count with SX_DIA_ND6=0)
  if (c.dia_n == 5 && ctx->dia_nd6) dia_go<spmv_dia_kernel<T, 5, Epi, FMA, V, Gather>>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
  else if (c.dia_n == 7 && ctx->dia_nd6) dia_go<spmv_dia_kernel<T, 7, Epi, FMA, V, Gather>>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
  else if (c.dia_n == 9 && ctx->dia_nd6) dia_go<spmv_dia_kernel<T, 9, Epi, FMA, V, Gather>>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
  else dia_go<spmv_dia_kernel<T, kDiaGeneric, Epi, FMA, V, Gather>>(ctx, c, vals, x, y, epi, ra, gat, offs, groups);
  return true;
}

// Short-row SpMV launch: K = 8, 12 or 16 by the longest row (monotone
// matrices only); false when rows are longer than 16.
template <typename T, class Epi, bool FMA, typename V = T, class Gather = GatherPlain<T>>
bool launch_short(sx_ctx ctx, const DevCsr& c, const V* vals, const T* x, T* y, Epi epi, const ReduceArea& ra,
                  int64_t blocks, Gather gat = Gather{}) {
  if (!c.monotone || c.max_row_len > 16) return false;
  auto go = [&](auto kern) {
    const int64_t grid = std::min<int64_t>(blocks, (int64_t)ctx->num_sms * 8);
    kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(c.indptr, c.indices, vals, x, y, c.nrows, (T*)ra.partials,
                                                      ra.counter, epi, gat);
  };
  if (c.max_row_len <= 8) go(spmv_short_kernel<T, 8, Epi, FMA, V, Gather>);
  else if (c.max_row_len <= 12) go(spmv_short_kernel<T, 12, Epi, FMA, V, Gather>);
  else go(spmv_short_kernel<T, 16, Epi, FMA, V, Gather>);
  return true;
}

template <typename T, int ITEMS, class Epi, class Gather, typename V>
void launch_pipe_gather_v(sx_ctx ctx, const DevCsr& c, const V* vals, const T* x, T* y, Epi epi, Gather gat,
                          const ReduceArea& ra, int64_t blocks) {
  constexpr auto kern = spmv_pipe_kernel<T, ITEMS, Epi, false, false, 1, V, Gather>;
  const int64_t grid = std::min<int64_t>(blocks, (int64_t)ctx->num_sms * resident_blocks<kern>());
  kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(c.indptr, c.indices, vals, x, y, c.nrows, blocks,
                                                    (T*)ra.partials, ra.counter, epi, nullptr, nullptr, gat);
}

// The register pipeline with a custom gather (fused solver steps); false
// when the matrix's chunks do not fit it.  HALF as in launch_csr.
template <typename T, class Epi, class Gather, bool HALF>
bool launch_pipe_gather(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi, Gather gat) {
  if (c.nrows <= 0) return true;
  if (!(c.monotone && c.max_chunk_nnz + 3 <= kBlock * 12)) return false;
  ReduceArea ra;
  const int64_t blocks = (c.nrows + kBlock - 1) / kBlock;
  if (ctx_reduce_area(ctx, blocks, &ra) != SX_OK) return false;
  const bool small = c.max_chunk_nnz + 3 <= kBlock * 8;
  bool done = false;
  if constexpr (HALF && sizeof(T) == 4) {
    if (c.dia_vals16)
      done = launch_dia<T, Epi, false, __half, Gather>(ctx, c, (const __half*)c.dia_vals16, x, y, epi, ra, blocks, gat);
  }
  if (!done) done = launch_dia<T, Epi, false, T, Gather>(ctx, c, (const T*)c.dia_vals, x, y, epi, ra, blocks, gat);
  if (!done && ctx->short_rows == 2) {
    if constexpr (HALF && sizeof(T) == 4) {
      if (c.vals16) done = launch_short<T, Epi, false, __half, Gather>(ctx, c, (const __half*)c.vals16, x, y, epi, ra, blocks, gat);
    }
    if (!done) done = launch_short<T, Epi, false, T, Gather>(ctx, c, (const T*)c.vals, x, y, epi, ra, blocks, gat);
  }
  if constexpr (HALF && sizeof(T) == 4) {
    if (!done && c.vals16) {
      if (small) launch_pipe_gather_v<T, 8>(ctx, c, (const __half*)c.vals16, x, y, epi, gat, ra, blocks);
      else launch_pipe_gather_v<T, 12>(ctx, c, (const __half*)c.vals16, x, y, epi, gat, ra, blocks);
      done = true;
    }
  }
  if (!done) {
    if (small) launch_pipe_gather_v<T, 8>(ctx, c, (const T*)c.vals, x, y, epi, gat, ra, blocks);
    else launch_pipe_gather_v<T, 12>(ctx, c, (const T*)c.vals, x, y, epi, gat, ra, blocks);
  }
  ctx->launches++;
  return cudaGetLastError() == cudaSuccess;
}

// register budget: 8 resident blocks per SM for FP32 with 8 items per thread
// (no spills; measured fastest on the 128^3 Laplacian), the compiler's
// choice otherwise (FP64 spills under a tighter budget)
template <typename T, int ITEMS, class Epi, bool FMA, bool C16>
void launch_pipe(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi, const ReduceArea& ra, int64_t blocks) {
  constexpr int kMinBlocks = (sizeof(T) == 4 && ITEMS == 8) ? 8 : 1;
  launch_pipe_minb<T, ITEMS, Epi, FMA, C16, kMinBlocks>(ctx, c, x, y, epi, ra, blocks);
}

// CSR SpMV with epilogue.  Must not allocate or synchronise: it runs inside
// stream capture.  The reduction area must already hold gridDim blocks.
// HALF: FP32 values may be read from the FP16 copy where one exists.
// The kernel launch_csr picks for a matrix (its decision order, as a name):
// keep in step with launch_csr below.
inline const char* spmv_kernel_name(sx_ctx ctx, const DevCsr& c, int w, bool fma, bool half_ok) {
  const bool pipe_fits = c.monotone && c.max_chunk_nnz + 3 <= kBlock * 12;
  const bool items8 = c.max_chunk_nnz + 3 <= kBlock * 8;
  if (c.nrows <= 0) return "none";
  if (ctx->dia && c.dia_n > 0 && c.dia_mask) {
    const bool h = half_ok && w == 4 && c.dia_vals16;
    if (ctx->dia_nd6 && ctx->dia_band) {
      const unsigned bm = dia_band_mask(c.dia_off, c.dia_n);
      if (c.dia_n == 9 && bm == 0x49u) return h ? "spmv_dia_kernel<ND=9, bands 3+3+3, FP16 values>" : "spmv_dia_kernel<ND=9, bands 3+3+3>";
      if (c.dia_n == 7 && bm == 0x67u) return h ? "spmv_dia_kernel<ND=7, bands 1+1+3+1+1, FP16 values>" : "spmv_dia_kernel<ND=7, bands 1+1+3+1+1>";
      if (c.dia_n == 5 && bm == 0x13u) return h ? "spmv_dia_kernel<ND=5, bands 1+3+1, FP16 values>" : "spmv_dia_kernel<ND=5, bands 1+3+1>";
      if (c.dia_n == 5 && bm == 0x09u) return h ? "spmv_dia_kernel<ND=5, bands 3+2, FP16 values>" : "spmv_dia_kernel<ND=5, bands 3+2>";
      if (c.dia_n == 5 && bm == 0x05u) return h ? "spmv_dia_kernel<ND=5, bands 2+3, FP16 values>" : "spmv_dia_kernel<ND=5, bands 2+3>";
    }
    if (c.dia_n == 5 && ctx->dia_nd6) return h ? "spmv_dia_kernel<ND=5, FP16 values>" : "spmv_dia_kernel<ND=5>";
    if (c.dia_n == 7 && ctx->dia_nd6) return h ? "spmv_dia_kernel<ND=7, FP16 values>" : "spmv_dia_kernel<ND=7>";
    if (c.dia_n == 9 && ctx->dia_nd6) return h ? "spmv_dia_kernel<ND=9, FP16 values>" : "spmv_dia_kernel<ND=9>";
    return h ? "spmv_dia_kernel<ND=16, FP16 values>" : "spmv_dia_kernel<ND=16>";
  }
  if (c.tile_row && ctx->win_mode == 1 && !pipe_fits && ctx->bin && c.sl_vals)
    return fma ? "spmv_sliced_kernel<FMA>" : "spmv_sliced_kernel";
  if (c.tile_row && (ctx->win_mode == 2 || (ctx->win_mode == 1 && !pipe_fits))) return "spmv_win_kernel";
  if (ctx->short_rows && (fma || (w == 4 && ctx->short_rows == 2)) && c.monotone && c.max_row_len <= 16)
    return c.max_row_len <= 8 ? "spmv_short_kernel<K=8>"
                              : (c.max_row_len <= 12 ? "spmv_short_kernel<K=12>" : "spmv_short_kernel<K=16>");
  if (pipe_fits && half_ok && w == 4 && c.vals16)
    return items8 ? "spmv_pipe_kernel<ITEMS=8, FP16 values>" : "spmv_pipe_kernel<ITEMS=12, FP16 values>";
  if (pipe_fits && c.col16 && ctx->col16)
    return items8 ? "spmv_pipe_kernel<ITEMS=8, 16-bit columns>" : "spmv_pipe_kernel<ITEMS=12, 16-bit columns>";
  if (pipe_fits) return items8 ? "spmv_pipe_kernel<ITEMS=8>" : "spmv_pipe_kernel<ITEMS=12>";
  if (c.monotone) return "spmv_stream_kernel";
  return "spmv_rowseq_kernel";
}

template <typename T, class Epi, bool FMA = false, bool HALF = false>
int launch_csr(sx_ctx ctx, const DevCsr& c, const T* x, T* y, Epi epi) {
  if (c.nrows <= 0) return SX_OK;
  ReduceArea ra;
  const int64_t blocks = (c.nrows + kBlock - 1) / kBlock;
  SX_CHECK(ctx_reduce_area(ctx, blocks, &ra));
  // every 256-row chunk fits the register pipeline: stencil-like matrices
  const bool pipe_fits = c.monotone && c.max_chunk_nnz + 3 <= kBlock * 12;
  bool done = false;
  // the diagonal layout first (stencil matrices: no column indices to read)
  if constexpr (HALF && sizeof(T) == 4) {
    if (c.dia_vals16) done = launch_dia<T, Epi, FMA, __half>(ctx, c, (const __half*)c.dia_vals16, x, y, epi, ra, blocks);
  }
  if (!done) done = launch_dia<T, Epi, FMA>(ctx, c, (const T*)c.dia_vals, x, y, epi, ra, blocks);
  // long rows: the sliced layout (coalesced loads whatever the row lengths,
  // all lanes busy on the thin FP64 pipe)
  if (!done && c.tile_row && ctx->win_mode == 1 && !pipe_fits)
    done = launch_sliced<T, Epi, FMA>(ctx, c, x, y, epi, ra, blocks);
  if (!done && c.tile_row && (ctx->win_mode == 2 || (ctx->win_mode == 1 && !pipe_fits))) {
    switch (ctx->win_shape) {
      case 1: done = launch_win<T, 1, Epi, FMA>(ctx, c, x, y, epi, ra, blocks); break;
      case 2: done = launch_win<T, 2, Epi, FMA>(ctx, c, x, y, epi, ra, blocks); break;
      default: done = launch_win<T, 0, Epi, FMA>(ctx, c, x, y, epi, ra, blocks); break;
    }
  }
  // short rows: the register-only kernel for FP64 with fused multiply-adds
  // (faster alone, equal inside the solvers); FP32 and exact FP64 keep the
  // pipeline, which is equal or faster inside the solvers' graphs
  // (SX_SHORT=2 extends it to FP32)
  if (!done && ctx->short_rows && (FMA || (sizeof(T) == 4 && ctx->short_rows == 2))) {
    bool half = false;
    if constexpr (HALF && sizeof(T) == 4) half = c.vals16 != nullptr;
    if constexpr (HALF && sizeof(T) == 4) {
      if (half) done = launch_short<T, Epi, FMA, __half>(ctx, c, (const __half*)c.vals16, x, y, epi, ra, blocks);
    }
    if (!done && !half) done = launch_short<T, Epi, FMA>(ctx, c, (const T*)c.vals, x, y, epi, ra, blocks);
  }
  if constexpr (HALF && sizeof(T) == 4) {
    if (!done && pipe_fits && c.vals16) {
      if (c.max_chunk_nnz + 3 <= kBlock * 8) launch_pipe_minb<T, 8, Epi, FMA, false, 1, __half>(ctx, c, x, y, epi, ra, blocks);
      else launch_pipe_minb<T, 12, Epi, FMA, false, 1, __half>(ctx, c, x, y, epi, ra, blocks);
      done = true;
    }
  }
  if (done) {
  } else if (pipe_fits && c.col16 && ctx->col16) {
    if (c.max_chunk_nnz + 3 <= kBlock * 8) launch_pipe<T, 8, Epi, FMA, true>(ctx, c, x, y, epi, ra, blocks);
    else launch_pipe<T, 12, Epi, FMA, true>(ctx, c, x, y, epi, ra, blocks);
  } else if (pipe_fits) {
    if (c.max_chunk_nnz + 3 <= kBlock * 8) launch_pipe<T, 8, Epi, FMA, false>(ctx, c, x, y, epi, ra, blocks);
    else launch_pipe<T, 12, Epi, FMA, false>(ctx, c, x, y, epi, ra, blocks);
  } else if (c.monotone) {
    spmv_stream_kernel<T, kSpmvItems, Epi, FMA><<<(unsigned)blocks, kBlock, 0, ctx->stream>>>(
        c.indptr, c.indices, (const T*)c.vals, x, y, c.nrows, (T*)ra.partials, ra.counter, epi);
  } else {
    spmv_rowseq_kernel<T, Epi><<<(unsigned)blocks, kBlock, 0, ctx->stream>>>(
        c.indptr, c.indices, (const T*)c.vals, x, y, c.nrows, (T*)ra.partials, ra.counter, epi);
  }
  ctx->launches++;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

template <typename T, class Body>
int launch_vec(sx_ctx ctx, int64_t n, Body body) {
  ReduceArea ra;
  const int g = vec_grid(ctx, n);
  SX_CHECK(ctx_reduce_area(ctx, g, &ra));
  vec_kernel<T, Body><<<g, kBlock, 0, ctx->stream>>>(n, (T*)ra.partials, ra.counter, body);
  ctx->launches++;
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

// EXACT = false (solver-internal use): FP64 CSR products use the FMA row
// sums, which halve the work of GB300's FP64 pipe and stay within a few ulp
// per row; EXACT = true reproduces the reference's per-row rounding.
template <typename T, class Epi, bool EXACT = false>
int launch_apply(sx_ctx ctx, sx_op op, const T* x, T* y, Epi epi) {
  constexpr bool kFma = !EXACT && sizeof(T) == 8;
  switch (op->kind) {
    case SX_OP_CSR:
    case SX_OP_SYM_CSR:  // the merged rows: stored row k, then column k below the diagonal
      return launch_csr<T, Epi, kFma>(ctx, op->csr, x, y, epi);
    case SX_OP_SUM: {
      // y = A x, w = B x, y = y + w with the epilogue
      SX_CHECK((launch_apply<T, EpiPlain<T>, EXACT>(ctx, op->left, x, y, EpiPlain<T>{})));
      SX_CHECK((launch_apply<T, EpiPlain<T>, EXACT>(ctx, op->right, x, (T*)op->work, EpiPlain<T>{})));
      ReduceArea ra;
      const int g = vec_grid(ctx, op->nrows);
      SX_CHECK(ctx_reduce_area(ctx, g, &ra));
      k_sum_epi<T, Epi><<<g, kBlock, 0, ctx->stream>>>(op->nrows, y, (const T*)op->work, (T*)ra.partials,
                                                        ra.counter, epi);
      ctx->launches++;
      SX_CUDA(cudaGetLastError());
      return SX_OK;
    }
    case SX_OP_PRODUCT: {
      // w = B x, then y = A w carries the epilogue
      SX_CHECK((launch_apply<T, EpiPlain<T>, EXACT>(ctx, op->right, x, (T*)op->work, EpiPlain<T>{})));
      return launch_apply<T, Epi, EXACT>(ctx, op->left, (const T*)op->work, y, epi);
    }
    case SX_OP_ZERO:
    case SX_OP_IDENTITY:
    case SX_OP_SCALED_IDENTITY:
    case SX_OP_DIAGONAL:
    case SX_OP_JACOBI: {
      ReduceArea ra;
      const int g = vec_grid(ctx, op->nrows);
      SX_CHECK(ctx_reduce_area(ctx, g, &ra));
      k_diag_apply<T, Epi><<<g, kBlock, 0, ctx->stream>>>(op->nrows, op->kind, (const T*)op->diag,
                                                          (T)op->scale, x, y, (T*)ra.partials,
                                                          ra.counter, epi);
      ctx->launches++;
      SX_CUDA(cudaGetLastError());
      return SX_OK;
    }
    case SX_OP_FSAI: {
      // y = G (G^T x): the second SpMV carries the epilogue; solver-internal
      // applies read a learned factor's FP16 values
      SX_CHECK(launch_csr<T, EpiPlain<T>, kFma, !EXACT>(ctx, op->transpose->csr, x, (T*)op->work, EpiPlain<T>{}));
      return launch_csr<T, Epi, kFma, !EXACT>(ctx, op->csr, (const T*)op->work, y, epi);
    }
    default: {
      // IC0 and host operators: apply, then run the epilogue over y
      SX_CHECK(apply_general(ctx, op, x, y));
      ReduceArea ra;
      const int g = vec_grid(ctx, op->nrows);
      SX_CHECK(ctx_reduce_area(ctx, g, &ra));
      k_epi_inplace<T, Epi><<<g, kBlock, 0, ctx->stream>>>(op->nrows, y, (T*)ra.partials,
                                                           ra.counter, epi);
      ctx->launches++;
      SX_CUDA(cudaGetLastError());
      return SX_OK;
    }
  }
}

}  // namespace sx
