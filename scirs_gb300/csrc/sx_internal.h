// Internal declarations shared by the translation units of the GB300 sparse
// library.  Nothing here is part of the C ABI (include/scirs_sparse.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "scirs_sparse.h"

namespace sx {

// ----------------------------------------------------------------- errors
int set_error(int code, const std::string& msg, uint64_t v0 = 0, uint64_t v1 = 0, uint64_t v2 = 0,
              uint64_t v3 = 0);
int clear_error();
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define SX_CUDA(...)                                                             \
  do {                                                                           \
    cudaError_t sx_e_ = (__VA_ARGS__);                                           \
    if (sx_e_ != cudaSuccess) return ::sx::cuda_fail(sx_e_, #__VA_ARGS__, __FILE__, __LINE__); \
  } while (0)

#define SX_CHECK(...)                   \
  do {                                  \
    int sx_rc_ = (__VA_ARGS__);         \
    if (sx_rc_ != SX_OK) return sx_rc_; \
  } while (0)

// Message codes of IterationResult.message (sx_message in the ABI).
enum : int {
  MSG_CONVERGED = 0,
  MSG_MAX_ITER = 1,
  MSG_NOT_PD = 2,
  MSG_CONVERGED_INITIAL = 3,
  MSG_BD_RHO = 4,
  MSG_BD_RHAT_V = 5,
  MSG_BD_ALPHA = 6,
  MSG_BD_TT = 7,
  MSG_BD_OMEGA = 8,
  MSG_BICG_PQ = 9,
  MSG_BICG_RHO = 10,
  MSG_CGS_RHO = 11,
  MSG_CGS_SIGMA = 12,
  MSG_QMR_INITIAL = 13,
  MSG_QMR_RHO = 14,
  MSG_QMR_PQ = 15,
  MSG_QMR_CONVERGED = 16,
  MSG_QMR_OMEGA = 17,
  MSG_QMR_MAX_ITER = 18,
  MSG_ZERO_RHS = 19,
  MSG_ZERO_RESIDUAL = 20,
};

// ------------------------------------------------------------ device CSR
// int32 row pointers and columns (nnz < 2^31), values of the handle dtype.
struct DevCsr {
  int64_t nrows = 0, ncols = 0, nnz = 0;
  int32_t* indptr = nullptr;   // nrows + 1
  int32_t* indices = nullptr;  // nnz
  void* vals = nullptr;        // nnz values
  bool has_sorted_indices = true;
  bool monotone = true;        // indptr non-decreasing
  int32_t max_row_len = 0;
  double mean_row_len = 0.0;
  int32_t max_chunk_nnz = 0;   // most nonzeros in any 256-row chunk
  // first row of every 256-entry unit of the nonzeros (units + 1 entries),
  // set for monotone matrices with indptr[0] == 0 and nnz > 0
  int32_t* tile_row = nullptr;
  int64_t units = 0;
  // rows ordered by length, longest first (a stable counting sort on
  // min(length, 4096)), for the sliced SpMV of long-row matrices
  int32_t* bin_perm = nullptr;
  // sliced layout: the rows in bin_perm order, in slices of 32 rows; slice s
  // stores position j of its row q at sl_base[s] + 32 j + q (columns and
  // values of the handle dtype), zero-padded to its longest row;
  // sl_len[32 s + q] = the length of that row (0 past the last row).
  // Slices [0, sl_big) hold a row longer than kSlBig entries, slices
  // [sl_short, sl_slices) only rows of at most kSlShort entries.
  int32_t* sl_cols = nullptr;
  void* sl_vals = nullptr;
  int64_t* sl_base = nullptr;  // sl_slices + 1
  int32_t* sl_len = nullptr;   // 32 * sl_slices
  int64_t sl_slices = 0, sl_big = 0, sl_short = 0;
  // compressed columns for the register-pipelined SpMV: col = chunk_base[r / 256]
  // + col16[k]; set when every 256-row chunk spans fewer than 65,536 columns
  uint16_t* col16 = nullptr;
  int32_t* chunk_base = nullptr;
  // FP16 copy of FP32 values (__half), read by solver-internal applies of a
  // learned factor; the exact API path keeps using vals
  void* vals16 = nullptr;
  // diagonal layout, set when the nonzeros lie on at most kDiaMax diagonals,
  // every row's columns strictly increase and the padding is small:
  // dia_vals[d * dia_ld + row] = the entry of `row` on diagonal d (offset
  // dia_off[d], ascending), zero where absent; bit d of dia_mask[row] says
  // whether the row stores that entry.  Ascending offsets are the storage
  // order of a sorted row, so a row's sum keeps the CSR order.
  int32_t dia_n = 0;
  int32_t dia_off[16] = {0};
  int64_t dia_ld = 0;
  void* dia_vals = nullptr;
  void* dia_vals16 = nullptr;  // FP16 copy, with vals16
  uint16_t* dia_mask = nullptr;
};
constexpr int kDiaMax = 16;

struct IC0Dev;   // defined in sx_ic0.cu
struct TriDev;   // ILU(0) / SSOR, defined in sx_ilu.cu
void tri_destroy(TriDev* p);
struct HostOp {
  sx_host_matvec_fn fn = nullptr;
  void* user = nullptr;
};

}  // namespace sx

struct sx_op_s {
  int kind = SX_OP_CSR;
  int dtype = SX_F64;
  int device = 0;
  int64_t nrows = 0, ncols = 0;
  sx::DevCsr csr;                     // CSR, and G for FSAI
  void* diag = nullptr;               // DIAGONAL: d; JACOBI: 1/d
  double scale = 1.0;                 // SCALED_IDENTITY
  sx_op_s* transpose = nullptr;       // cached transpose (rmatvec, FSAI's G^T)
  sx::IC0Dev* ic0 = nullptr;
  sx::TriDev* tri = nullptr;          // ILU0 / SSOR
  sx::HostOp host;
  void* work = nullptr;               // per-operator temporary vector (FSAI: G^T x;
                                      // SUM: B x; PRODUCT: B x)
  sx_op_s* left = nullptr;            // SUM / PRODUCT operands, borrowed
  sx_op_s* right = nullptr;
  sx_op_s* sym_low = nullptr;         // SYM_CSR: the stored lower triangle (owned);
                                      // csr holds the merged rows applied by SpMV
  uint64_t serial = 0;                // unique id, keys the solver graph cache
};

struct sx_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  uint64_t launches = 0;
  // grow-only scratch; synchronises the stream before it is replaced
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // pinned host staging for scalar readback
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  // reduction partials (3 slots per block) and the last-block counter
  void* red_partials = nullptr;
  size_t red_bytes = 0;
  unsigned int* red_counter = nullptr;
  // solver workspaces and instantiated graphs (sx_krylov.cu)
  void* solver_cache = nullptr;
  // SpMV kernel choice from SX_WIN: 0 never the windowed kernel, 1 (default)
  // the windowed kernel for matrices whose 256-row chunks are too long for
  // the register pipeline, 2 the windowed kernel whenever it applies;
  // SX_WIN_SHAPE=0|1|2 picks its window shape
  int win_mode = 1;
  // SX_COL16=1: the register-pipelined SpMV reads the 16-bit column copy
  // where it exists (fewer bytes, but the decode costs registers and the
  // kernel is latency bound: slower on GB300, off by default)
  bool col16 = false;
  // SX_MX_FUSED=0: the residual-replacement loop runs the plain CG kernels
  // instead of its fused iteration
  bool mx_unfused = false;
  // matrices whose rows all hold at most 16 entries use the register-only
  // short-row SpMV: 1 (default) for FP64 with fused multiply-adds, 2 also
  // for FP32, 0 never (SX_SHORT)
  int short_rows = 1;
  // diagonal layout (SX_DIA): 0 never built or used; 1 (default) used for
  // every matrix that has it
  int dia = 1;
  // SX_DIA_ND6=0: every diagonal count takes the generic (runtime-count)
  // diagonal kernel instead of the exact-count ones
  bool dia_nd6 = true;
  // SX_DIA_BAND=0: the exact-count kernels read x per diagonal, never per
  // band of adjacent diagonals
  bool dia_band = true;
  // SX_PDL=0: diagonal-layout SpMVs launched without programmatic dependent
  // launch (each waits for the previous kernel to finish before starting)
  bool pdl = true;
  // SX_BIN=0: long-row matrices take the windowed SpMV instead of the
  // sliced one
  bool bin = true;
  // limit of one dependency wait of the triangular factorisations and
  // sweeps (IC(0), ILU(0), SSOR), in nanoseconds: a wait that runs longer
  // gives up and the call reports SX_ERR_DEVICE_TIMEOUT
  unsigned long long wait_ns = 2000000000ull;
  // sx_ctx_set_cg_recurrence: CG with a diagonal preconditioner carries A p
  // by the recurrence q = A z + beta q (two kernels per iteration)
  bool cg_recurrence = false;
  // autotuner results of this context: a kernel family and a key made of
  // size statistics -> the chosen launch shape (sx_tune.cuh)
  std::map<uint64_t, uint32_t> tuned;
  int win_shape = 0;
};

namespace sx {

int ctx_scratch(sx_ctx ctx, size_t bytes, void** out);
int ctx_pinned(sx_ctx ctx, size_t bytes, void** out);
inline size_t elt_size(int dtype) { return dtype == SX_F64 ? 8 : 4; }
inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Allocation helpers that record the CUDA error.
int dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
// the streams whose queued work a freed block waits for before its reuse
void mem_cache_register_stream(int device, cudaStream_t s);
void mem_cache_unregister_stream(int device, cudaStream_t s);

// Upload host-side CSR arrays (already validated, int32) into a DevCsr and
// compute row statistics.
// w: bytes per value (4 or 8) to also build the diagonal layout; 0 skips it
int csr_finalize_stats(sx_ctx ctx, DevCsr& c, int w = 0);
int csr_prepare_dia(sx_ctx ctx, DevCsr& c, int w);
// FP16 copy of an FP32 CSR's values (c.vals16)
int csr_make_half(sx_ctx ctx, DevCsr& c);
// a process-unique operator serial (keys of the solvers' graph caches)
uint64_t next_op_serial();
// destroys the solvers' cached graphs (sx_krylov.cu); called before a
// buffer that captured graphs reference is reallocated
void solver_graphs_drop(sx_ctx ctx);
constexpr int kUnit = 256;  // nonzeros per tile_row entry
constexpr int kBinLong = 32;       // a row longer than this makes a long-row matrix (sliced SpMV)
constexpr int kBinBuckets = 4096;  // the length order's key is min(length, kBinBuckets)
constexpr int kSlBig = 256;        // sliced layout: big slices hold a row longer than this
constexpr int kSlShort = 4;        // sliced layout: short slices hold rows of at most this
// builds what the context's SpMV choice can use: c.tile_row for the
// windowed SpMV, the row order and sliced layout for long-row matrices (w =
// value bytes, 4 or 8; none for w = 0), and (SX_COL16=1, where the column
// spans allow) c.col16 / c.chunk_base for the register pipeline (allocates
// and synchronises)
int csr_prepare_tiles(sx_ctx ctx, DevCsr& c, int w);
// frees the row order and the sliced layout
void free_sliced(DevCsr& c);


// ------------------------------------------------------------ kernels API
// Plain device SpMV entry used by the ABI (y = A x, device pointers).
int spmv_device(sx_ctx ctx, sx_op a, const void* x, void* y, unsigned flags);

// y = op(x) for operators whose apply is more than one kernel (IC0, FSAI,
// host callbacks).  Enqueued on ctx->stream; no allocation, no sync except
// for host callbacks.
int apply_general(sx_ctx ctx, sx_op op, const void* x, void* y);

// Exclusive scan of m int32 counts into out[0..m] (synchronises the stream).
int exclusive_scan_i32(sx_ctx ctx, const int32_t* in, int64_t m, int32_t* out);

// Abort flag of an IC(0) operator's bounded waits -> SX_ERR_DEVICE_TIMEOUT.
int ic0_health(sx_ctx ctx, sx_op op);
int ctx_set_wait_limit(sx_ctx ctx, uint64_t ns);
int wait_selftest(sx_ctx ctx, uint64_t* waited_ns);

// Cached transpose of a CSR operator (rmatvec, FSAI's G^T).
int ensure_transpose(sx_ctx ctx, sx_op a);
int csr_transpose_internal(sx_ctx ctx, sx_op a, sx_op* out, bool stats = true);
int fsai_adopt(sx_ctx ctx, sx_op g, sx_op* out, sx_op gt = nullptr);  // takes g (and gt: G^T, else computed)
sx_op csr_op_adopt(sx_ctx ctx, int dtype, DevCsr& c);  // takes c
int sym_half_spmv(sx_ctx ctx, sx_op a, const void* x, void* y);  // sx_sym.cu
// rows in dependency-level order (forward: on the rows j < i of the pattern;
// backward: on j > i), on the device (sx_ic0.cu)
int level_order(sx_ctx ctx, const DevCsr& c, bool forward, int32_t** out);
// ILU(0) / SSOR (sx_ilu.cu): apply, and the abort flag of their waits
int tri_apply(sx_ctx ctx, sx_op op, const void* x, void* y);
int* tri_ctl(sx_op op);
void destroy_op_internal(sx_op op);

// Grid geometry for the vector kernels (fixed per device -> deterministic
// reductions).
int vec_grid(sx_ctx ctx, int64_t n);

// Counter/partials area used by every fused reduction launch: it must be
// zero-initialised once and is left zeroed by the finalizing block.
struct ReduceArea {
  double* partials = nullptr;   // 3 * max_blocks doubles (or floats)
  unsigned int* counter = nullptr;
  int max_blocks = 0;
};
int ctx_reduce_area(sx_ctx ctx, int64_t blocks, ReduceArea* out);

}  // namespace sx
