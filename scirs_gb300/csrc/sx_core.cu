// Core of the GB300 sparse library: errors, contexts, operator handles,
// device CSR construction / validation / transpose, and the matvec entry
// points of the C ABI (include/scirs_sparse.h).
//
// CSR construction on the device reproduces a stable sort by (row, col)
// without a global sort: entries are counted per row, scattered into their
// row's slot range in any order with the key (col << 32 | original index),
// and each row is then sorted by that key.  Keys are unique, so the result
// is exactly the order a stable sort on (row, col) gives
// (CsrMatrix::new, scirs2-sparse/src/csr.rs:129; CsrArray::from_triplets,
// csr_array.rs:193).  The transpose uses the same machinery with the key
// (storage position << 32 | row), which reproduces the counting sort of
// CsrMatrix::transpose (csr.rs:289-326).

#include <algorithm>
#include <limits>
#include <atomic>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_fp16.h>

#include "sx_internal.h"
#include "sx_kernels.cuh"

namespace sx {

// ------------------------------------------------------------------ errors
static thread_local sx_error_info g_err = {0, 0, 0, 0, 0, {0}};

int set_error(int code, const std::string& msg, uint64_t v0, uint64_t v1, uint64_t v2,
              uint64_t v3) {
  g_err.code = code;
  g_err.v0 = v0; g_err.v1 = v1; g_err.v2 = v2; g_err.v3 = v3;
  std::snprintf(g_err.message, sizeof(g_err.message), "%s", msg.c_str());
  return code;
}
int clear_error() {
  g_err.code = 0;
  g_err.message[0] = 0;
  return SX_OK;
}
int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char buf[400];
  std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e,
                cudaGetErrorString(e), what, file, line);
  if (e == cudaErrorMemoryAllocation) return set_error(SX_ERR_OUT_OF_MEMORY, buf);
  return set_error(SX_ERR_CUDA, buf);
}

static std::string dim_msg(uint64_t expected, uint64_t found) {
  return "Dimension mismatch: expected " + std::to_string(expected) + ", found " +
         std::to_string(found);
}
static int err_dim(uint64_t expected, uint64_t found) {
  return set_error(SX_ERR_DIMENSION_MISMATCH, dim_msg(expected, found), expected, found);
}
static int err_value(const std::string& s) { return set_error(SX_ERR_VALUE, "Value error: " + s); }
static int err_incons(const std::string& s) {
  return set_error(SX_ERR_INCONSISTENT_DATA, "Inconsistent data: " + s);
}
static int err_oob(uint64_t r, uint64_t c, uint64_t sr, uint64_t sc) {
  return set_error(SX_ERR_INDEX_OUT_OF_BOUNDS,
                   "Index (" + std::to_string(r) + ", " + std::to_string(c) +
                       ") out of bounds for array with shape (" + std::to_string(sr) + ", " +
                       std::to_string(sc) + ")",
                   r, c, sr, sc);
}
static int err_cast(uint64_t v) {
  return set_error(SX_ERR_INDEX_CAST_OVERFLOW,
                   "Index value " + std::to_string(v) +
                       " cannot be represented in the target type i32",
                   v);
}
// index_dtype.rs:109-170 reports the first value, in array order, that does
// not fit the target type.  Called only when a dimension exceeds i32, on
// host index arrays: returns the first entry above i32::MAX, or 0.
static uint64_t first_cast_overflow(const uint64_t* a, uint64_t n) {
  for (uint64_t k = 0; k < n; ++k)
    if (a[k] > (uint64_t)INT32_MAX) return a[k];
  return 0;
}

static int err_arg(const char* what) {
  return set_error(SX_ERR_INVALID_ARGUMENT, std::string("Invalid argument: ") + what);
}

// ------------------------------------------------------------ block cache
// Freed device blocks are kept for reuse rather than returned through
// cudaFree (which waits for the whole device) and taken again from
// cudaMalloc: one learned-preconditioner setup frees and allocates about
// sixty blocks, 4 ms of a 100 ms solve when each goes to the driver.
//
// A block freed while work queued on the library's streams may still use it
// carries one event per stream registered on its device (every context's
// stream), recorded at the free; it is handed out again only once all of
// them have completed (cudaEventQuery: the allocation never waits; a block
// still in use is skipped and cudaMalloc serves the request).  At most
// kCacheBytes per device are held (blocks above kCacheMaxBlock go straight
// back to the driver); a failed cudaMalloc empties the device's cache and
// tries once more.  Blocks freed while one of the device's streams is being
// captured go back to cudaFree as before.  SX_MEM_CACHE=0 turns the cache
// off; sx_mem_cache_trim() returns every held block to the driver.
namespace {
constexpr size_t kCacheBytes = (size_t)4 << 30;
constexpr size_t kCacheMaxBlock = (size_t)1 << 30;

struct CachedBlock {
  void* p;
  size_t bytes;
  std::vector<cudaEvent_t> evs;
};

struct BlockCache {
  std::mutex mu;
  bool init = false, on = true;
  std::unordered_map<void*, std::pair<size_t, int>> live;         // block -> (bytes, device)
  std::multimap<std::pair<int, size_t>, CachedBlock> blocks;       // (device, bytes) -> block
  std::map<int, size_t> held;                                      // device -> bytes held
  std::vector<std::pair<int, cudaStream_t>> streams;               // registered context streams
  std::map<int, std::vector<cudaEvent_t>> spare;                   // device -> unused events
};

// never destroyed: blocks may be freed from static destructors at exit
BlockCache& block_cache() {
  static BlockCache* c = new BlockCache();
  return *c;
}

// sizes served: up to 1 MiB a power of two (at least 1 KiB), above that a
// multiple of 2 MiB, so that repeated requests of one array size meet
size_t cache_round(size_t bytes) {
  if (bytes <= ((size_t)1 << 20)) {
    size_t r = 1024;
    while (r < bytes) r <<= 1;
    return r;
  }
  return align_up(bytes, (size_t)2 << 20);
}

bool events_done(const CachedBlock& b) {
  for (cudaEvent_t e : b.evs)
    if (cudaEventQuery(e) != cudaSuccess) return false;
  return true;
}

// caller holds mu; the block's events go back to the device's spare list
void recycle_events(BlockCache& bc, int dev, CachedBlock& b) {
  auto& sp = bc.spare[dev];
  sp.insert(sp.end(), b.evs.begin(), b.evs.end());
  b.evs.clear();
}

// returns the device's held blocks to the driver (cudaFree waits for the
// device first); caller holds mu
void cache_release_device(BlockCache& bc, int dev) {
  for (auto it = bc.blocks.lower_bound({dev, 0}); it != bc.blocks.end() && it->first.first == dev;) {
    recycle_events(bc, dev, it->second);
    cudaFree(it->second.p);
    it = bc.blocks.erase(it);
  }
  bc.held[dev] = 0;
}

void cache_init(BlockCache& bc) {
  if (bc.init) return;
  bc.init = true;
  if (const char* t = std::getenv("SX_MEM_CACHE")) bc.on = std::strcmp(t, "0") != 0;
}
}  // namespace

void mem_cache_register_stream(int device, cudaStream_t s) {
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lk(bc.mu);
  bc.streams.emplace_back(device, s);
}

void mem_cache_unregister_stream(int device, cudaStream_t s) {
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lk(bc.mu);
  for (auto it = bc.streams.begin(); it != bc.streams.end(); ++it)
    if (it->first == device && it->second == s) {
      bc.streams.erase(it);
      return;
    }
}

// Every device array carries 64 bytes of slack past its end: the windowed
// SpMV's 16-byte copies may read up to 15 bytes past the last element.
int dev_alloc(void** p, size_t bytes) {
  *p = nullptr;
  const size_t want = cache_round(align_up(bytes, 16) + 64);
  int dev = 0;
  SX_CUDA(cudaGetDevice(&dev));
  BlockCache& bc = block_cache();
  {
    std::lock_guard<std::mutex> lk(bc.mu);
    cache_init(bc);
    if (bc.on) {
      // the smallest held block that fits, at most 1/8 larger, whose users
      // have finished
      const size_t most = want + want / 8;
      for (auto it = bc.blocks.lower_bound({dev, want});
           it != bc.blocks.end() && it->first.first == dev && it->first.second <= most; ++it) {
        if (!events_done(it->second)) continue;
        *p = it->second.p;
        const size_t got = it->second.bytes;
        recycle_events(bc, dev, it->second);
        bc.blocks.erase(it);
        bc.held[dev] -= got;
        bc.live[*p] = {got, dev};
        return SX_OK;
      }
    }
  }
  cudaError_t e = cudaMalloc(p, want);
  if (e == cudaErrorMemoryAllocation) {
    (void)cudaGetLastError();
    {
      std::lock_guard<std::mutex> lk(bc.mu);
      cache_release_device(bc, dev);
    }
    e = cudaMalloc(p, want);
  }
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
  }
  std::lock_guard<std::mutex> lk(bc.mu);
  bc.live[*p] = {want, dev};
  return SX_OK;
}

void dev_free(void* p) {
  if (!p) return;
  BlockCache& bc = block_cache();
  std::unique_lock<std::mutex> lk(bc.mu);
  cache_init(bc);
  auto it = bc.live.find(p);
  if (it == bc.live.end()) {  // not from dev_alloc
    lk.unlock();
    cudaFree(p);
    return;
  }
  const size_t bytes = it->second.first;
  const int dev = it->second.second;
  bc.live.erase(it);
  bool keep = bc.on && bytes <= kCacheMaxBlock;
  for (const auto& s : bc.streams) {
    if (!keep) break;
    if (s.first != dev) continue;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s.second, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) keep = false;
  }
  if (!keep) {
    lk.unlock();
    cudaFree(p);
    return;
  }
  int cur = dev;
  cudaGetDevice(&cur);
  if (cur != dev) cudaSetDevice(dev);
  CachedBlock b{p, bytes, {}};
  auto& sp = bc.spare[dev];
  for (const auto& s : bc.streams) {
    if (s.first != dev) continue;
    cudaEvent_t e = nullptr;
    if (!sp.empty()) {
      e = sp.back();
      sp.pop_back();
    } else if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      keep = false;
      break;
    }
    b.evs.push_back(e);
    if (cudaEventRecord(e, s.second) != cudaSuccess) {
      keep = false;
      break;
    }
  }
  if (!keep) {
    (void)cudaGetLastError();
    recycle_events(bc, dev, b);
    if (cur != dev) cudaSetDevice(cur);
    lk.unlock();
    cudaFree(p);
    return;
  }
  bc.blocks.emplace(std::make_pair(dev, bytes), std::move(b));
  bc.held[dev] += bytes;
  // over the limit: the largest finished blocks go back to the driver
  for (auto jt = bc.blocks.lower_bound({dev + 1, 0}); bc.held[dev] > kCacheBytes && jt != bc.blocks.begin();) {
    --jt;
    if (jt->first.first != dev) break;
    if (!events_done(jt->second)) continue;
    recycle_events(bc, dev, jt->second);
    cudaFree(jt->second.p);
    bc.held[dev] -= jt->first.second;
    jt = bc.blocks.erase(jt);
  }
  if (cur != dev) cudaSetDevice(cur);
}

int ctx_scratch(sx_ctx ctx, size_t bytes, void** out) {
  if (bytes > ctx->scratch_bytes) {
    if (ctx->scratch) {
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      dev_free(ctx->scratch);
      ctx->scratch = nullptr;
      ctx->scratch_bytes = 0;
    }
    size_t want = std::max(bytes, (size_t)1 << 20);
    SX_CHECK(dev_alloc(&ctx->scratch, want));
    ctx->scratch_bytes = want;
  }
  *out = ctx->scratch;
  return SX_OK;
}

int ctx_pinned(sx_ctx ctx, size_t bytes, void** out) {
  if (bytes > ctx->pinned_bytes) {
    if (ctx->pinned) {
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      cudaFreeHost(ctx->pinned);
      ctx->pinned = nullptr;
    }
    size_t want = std::max(bytes, (size_t)4096);
    SX_CUDA(cudaMallocHost(&ctx->pinned, want));
    ctx->pinned_bytes = want;
  }
  *out = ctx->pinned;
  return SX_OK;
}

int vec_grid(sx_ctx ctx, int64_t n) {
  int64_t want = (n + kBlock - 1) / kBlock;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

int ctx_reduce_area(sx_ctx ctx, int64_t blocks, ReduceArea* out) {
  size_t need = (size_t)std::max<int64_t>(blocks, 1) * 3 * sizeof(double);
  if (!ctx->red_counter) {
    void* c = nullptr;
    SX_CHECK(dev_alloc(&c, 256));
    SX_CUDA(cudaMemset(c, 0, 256));
    ctx->red_counter = (unsigned int*)c;
  }
  if (need > ctx->red_bytes) {
    if (ctx->red_partials) {
      SX_CUDA(cudaStreamSynchronize(ctx->stream));
      // captured solver graphs hold the old address
      solver_graphs_drop(ctx);
      dev_free(ctx->red_partials);
      ctx->red_partials = nullptr;
      ctx->red_bytes = 0;
    }
    size_t want = std::max(need, (size_t)1 << 20);
    SX_CHECK(dev_alloc(&ctx->red_partials, want));
    ctx->red_bytes = want;
  }
  out->partials = (double*)ctx->red_partials;
  out->counter = ctx->red_counter;
  out->max_blocks = (int)(ctx->red_bytes / (3 * sizeof(double)));
  return SX_OK;
}

// ============================================================ construction
namespace {

constexpr uint64_t kI32Max = 2147483647ull;

// Validation and narrowing of triplets.  flags[0]: some row >= nrows,
// flags[1]: some col >= ncols; first_bad: smallest k with either.
__global__ void k_triplet_check(const uint64_t* __restrict__ rows, const uint64_t* __restrict__ cols,
                                int64_t nnz, uint64_t nrows, uint64_t ncols, int32_t* rows32,
                                int32_t* cols32, int* flags, unsigned long long* first_bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    uint64_t r = rows[k], c = cols[k];
    bool br = r >= nrows, bc = c >= ncols;
    if (br) flags[0] = 1;
    if (bc) flags[1] = 1;
    if (br || bc) atomicMin(first_bad, (unsigned long long)k);
    rows32[k] = br ? 0 : (int32_t)r;
    cols32[k] = bc ? 0 : (int32_t)c;
  }
}

__global__ void k_count(const int32_t* __restrict__ key, int64_t n, int32_t* cnt) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    atomicAdd(cnt + key[k], 1);
}
// *out = max(cnt[0 .. m)), *out zero on entry
__global__ void k_max_count(const int32_t* __restrict__ cnt, int64_t m, int32_t* out) {
  int32_t v = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += stride) v = max(v, cnt[k]);
  v = max(v, __shfl_xor_sync(0xffffffffu, v, 16));
  v = max(v, __shfl_xor_sync(0xffffffffu, v, 8));
  v = max(v, __shfl_xor_sync(0xffffffffu, v, 4));
  v = max(v, __shfl_xor_sync(0xffffffffu, v, 2));
  v = max(v, __shfl_xor_sync(0xffffffffu, v, 1));
  if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(out, v);
}

// Exclusive scan, three phases: block sums, scan of the sums (recursive),
// block-local scan plus offset.  in has m entries; out has m + 1.
constexpr int kScanItems = 8;
constexpr int kScanTile = kBlock * kScanItems;

__global__ void k_scan_block_sums(const int32_t* __restrict__ in, int64_t m, int32_t* sums) {
  __shared__ int32_t sh[kWarps];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int32_t s = 0;
  for (int j = 0; j < kScanItems; ++j) {
    int64_t i = base + (int64_t)j * kBlock + threadIdx.x;
    if (i < m) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t t = 0;
    for (int w = 0; w < kWarps; ++w) t += sh[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void k_scan_apply(const int32_t* __restrict__ in, int64_t m,
                             const int32_t* __restrict__ offs, int32_t* out) {
  __shared__ int32_t tile[kScanTile];
  __shared__ int32_t wsum[kWarps];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  for (int j = 0; j < kScanItems; ++j) {
    int64_t i = base + (int64_t)j * kBlock + threadIdx.x;
    tile[j * kBlock + threadIdx.x] = i < m ? in[i] : 0;
  }
  __syncthreads();
  // each thread scans kScanItems consecutive entries
  int32_t loc[kScanItems];
  int32_t run = 0;
  for (int j = 0; j < kScanItems; ++j) {
    loc[j] = run;
    run += tile[threadIdx.x * kScanItems + j];
  }
  // exclusive scan of thread totals across the block
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t v = run;
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  int32_t wo = 0;
  for (int q = 0; q < w; ++q) wo += wsum[q];
  int32_t texcl = wo + v - run + offs[blockIdx.x];
  __syncthreads();
  for (int j = 0; j < kScanItems; ++j) tile[threadIdx.x * kScanItems + j] = texcl + loc[j];
  __syncthreads();
  for (int j = 0; j < kScanItems; ++j) {
    int64_t i = base + (int64_t)j * kBlock + threadIdx.x;
    if (i < m) out[i] = tile[j * kBlock + threadIdx.x];
  }
}

__global__ void k_scan_total(const int32_t* __restrict__ in, int64_t m, int32_t* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) out[m] = (m > 0 ? out[m - 1] + in[m - 1] : 0);
}

}  // namespace

// exclusive scan of m int32 counts into out[0..m]; temporaries from cudaMalloc
static int scan_exclusive(sx_ctx ctx, const int32_t* in, int64_t m, int32_t* out) {
  if (m <= 0) {
    SX_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), ctx->stream));
    return SX_OK;
  }
  int64_t nb = (m + kScanTile - 1) / kScanTile;
  int32_t *sums = nullptr, *offs = nullptr;
  SX_CHECK(dev_alloc((void**)&sums, nb * sizeof(int32_t)));
  SX_CHECK(dev_alloc((void**)&offs, (nb + 1) * sizeof(int32_t)));
  k_scan_block_sums<<<(unsigned)nb, kBlock, 0, ctx->stream>>>(in, m, sums);
  ctx->launches++;
  int rc = SX_OK;
  if (nb == 1) {
    cudaMemsetAsync(offs, 0, sizeof(int32_t), ctx->stream);
  } else {
    rc = scan_exclusive(ctx, sums, nb, offs);
  }
  if (rc == SX_OK) {
    k_scan_apply<<<(unsigned)nb, kBlock, 0, ctx->stream>>>(in, m, offs, out);
    k_scan_total<<<1, 32, 0, ctx->stream>>>(in, m, out);
    ctx->launches += 2;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "scan", __FILE__, __LINE__);
  }
  dev_free(sums);
  dev_free(offs);
  return rc;
}

int exclusive_scan_i32(sx_ctx ctx, const int32_t* in, int64_t m, int32_t* out) {
  return scan_exclusive(ctx, in, m, out);
}

namespace {

// Scatter triplet k into its row's slot range with key (col << 32 | k).
__global__ void k_scatter_rows(const int32_t* __restrict__ rows32, const int32_t* __restrict__ cols32,
                               int64_t nnz, const int32_t* __restrict__ indptr, int32_t* cursor,
                               unsigned long long* keys) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    int32_t r = rows32[k];
    int32_t pos = indptr[r] + atomicAdd(cursor + r, 1);
    keys[pos] = ((unsigned long long)(uint32_t)cols32[k] << 32) | (unsigned long long)k;
  }
}

// Transpose scatter: one thread per row walks its entries; key
// (storage position << 32 | row).
__global__ void k_scatter_cols(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                               int64_t nrows, const int32_t* __restrict__ tptr, int32_t* cursor,
                               unsigned long long* keys) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    for (int32_t k = indptr[r]; k < indptr[r + 1]; ++k) {
      int32_t c = indices[k];
      int32_t pos = tptr[c] + atomicAdd(cursor + c, 1);
      keys[pos] = ((unsigned long long)(uint32_t)k << 32) | (unsigned long long)(uint32_t)r;
    }
  }
}

// Row-length buckets for the per-row sort.
__global__ void k_bucket_rows(const int32_t* __restrict__ ptr, int64_t m, int32_t* lists,
                              int32_t* counts, int64_t cap) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += stride) {
    int32_t L = ptr[r + 1] - ptr[r];
    int b = L <= 1 ? -1 : (L <= 32 ? 0 : (L <= 2048 ? 1 : 2));
    if (b >= 0) {
      int32_t slot = atomicAdd(counts + b, 1);
      lists[(int64_t)b * cap + slot] = (int32_t)r;
    }
  }
}

// rows of length <= 32: one thread, insertion sort in registers/local memory
__global__ void k_sort_small(const int32_t* __restrict__ ptr, const int32_t* __restrict__ list,
                             const int32_t* __restrict__ count, unsigned long long* keys) {
  int32_t n = *count;
  for (int32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int32_t r = list[t];
    int32_t s = ptr[r], L = ptr[r + 1] - s;
    unsigned long long v[32];
    for (int i = 0; i < L; ++i) v[i] = keys[s + i];
    for (int i = 1; i < L; ++i) {
      unsigned long long x = v[i];
      int j = i - 1;
      while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
      v[j + 1] = x;
    }
    for (int i = 0; i < L; ++i) keys[s + i] = v[i];
  }
}

// bitonic sort of one segment of length L <= CAP in shared memory
template <int CAP>
__device__ void block_bitonic(unsigned long long* sm, unsigned long long* g, int32_t L) {
  for (int i = threadIdx.x; i < CAP; i += blockDim.x) sm[i] = i < L ? g[i] : ~0ull;
  __syncthreads();
  for (int k = 2; k <= CAP; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < CAP; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          unsigned long long a = sm[i], b = sm[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) { sm[i] = b; sm[ixj] = a; }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < L; i += blockDim.x) g[i] = sm[i];
  __syncthreads();
}

__global__ void k_sort_mid(const int32_t* __restrict__ ptr, const int32_t* __restrict__ list,
                           const int32_t* __restrict__ count, unsigned long long* keys) {
  __shared__ unsigned long long sm[2048];
  int32_t n = *count;
  for (int32_t t = blockIdx.x; t < n; t += gridDim.x) {
    int32_t r = list[t];
    int32_t s = ptr[r], L = ptr[r + 1] - s;
    block_bitonic<2048>(sm, keys + s, L);
  }
}

// Long segments: sort chunks of 2048 in shared memory, then merge runs
// pairwise in global memory.  Keys are unique, so the output position of
// an element is its rank in its own run plus the number of smaller keys in
// the partner run.
__global__ void k_sort_chunks(unsigned long long* keys, int32_t L) {
  __shared__ unsigned long long sm[2048];
  int32_t c0 = blockIdx.x * 2048;
  if (c0 >= L) return;
  block_bitonic<2048>(sm, keys + c0, min(2048, L - c0));
}

__global__ void k_merge_pass(const unsigned long long* __restrict__ in, unsigned long long* out,
                             int32_t L, int32_t width) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += stride) {
    int32_t run = (int32_t)(i / width);
    int32_t pair = run >> 1;
    int32_t a0 = pair * 2 * width;
    int32_t a1 = min(L, a0 + width);
    int32_t b0 = a1, b1 = min(L, a0 + 2 * width);
    unsigned long long v = in[i];
    int32_t lo, hi;
    if ((run & 1) == 0) { lo = b0; hi = b1; } else { lo = a0; hi = a1; }
    // count of keys < v in the partner run
    int32_t l = lo, h = hi;
    while (l < h) {
      int32_t mid = (l + h) >> 1;
      if (in[mid] < v) l = mid + 1; else h = mid;
    }
    int32_t rank_other = l - lo;
    int32_t rank_own = (int32_t)i - ((run & 1) == 0 ? a0 : b0);
    out[a0 + rank_own + rank_other] = v;
  }
}

}  // namespace

// Sort each segment [ptr[r], ptr[r+1]) of keys ascending.
// Host copy of the segment pointers, taken only when some segment is
// longer than the in-register sorts handle (cnt[m] is free scratch: the
// counts use cnt[0 .. m)); empty otherwise.  Synchronises the stream.
static int long_segment_ptr(sx_ctx ctx, int32_t* cnt, int64_t m, const int32_t* d_ptr,
                            std::vector<int32_t>& h_ptr) {
  h_ptr.clear();
  int32_t maxc = 0;
  cudaMemsetAsync(cnt + m, 0, 4, ctx->stream);
  if (m > 0) {
    k_max_count<<<vec_grid(ctx, m), kBlock, 0, ctx->stream>>>(cnt, m, cnt + m);
    ctx->launches++;
  }
  cudaMemcpyAsync(&maxc, cnt + m, 4, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "segment lengths", __FILE__, __LINE__);
  if (maxc > 2048) {
    h_ptr.resize(m + 1);
    cudaMemcpyAsync(h_ptr.data(), d_ptr, (m + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "segment pointers", __FILE__, __LINE__);
  }
  return SX_OK;
}

// h_ptr: the host segment pointers when a segment is longer than 2,048,
// else empty
static int segmented_sort(sx_ctx ctx, const int32_t* d_ptr, int64_t m, unsigned long long* keys,
                          const std::vector<int32_t>& h_ptr) {
  if (m <= 0) return SX_OK;
  int32_t *lists = nullptr, *counts = nullptr;
  SX_CHECK(dev_alloc((void**)&lists, 3 * (size_t)m * sizeof(int32_t)));
  SX_CHECK(dev_alloc((void**)&counts, 4 * sizeof(int32_t)));
  cudaMemsetAsync(counts, 0, 4 * sizeof(int32_t), ctx->stream);
  int g = vec_grid(ctx, m);
  k_bucket_rows<<<g, kBlock, 0, ctx->stream>>>(d_ptr, m, lists, counts, m);
  k_sort_small<<<g, kBlock, 0, ctx->stream>>>(d_ptr, lists, counts, keys);
  k_sort_mid<<<ctx->num_sms * 4, kBlock, 0, ctx->stream>>>(d_ptr, lists + m, counts + 1, keys);
  ctx->launches += 3;
  int rc = SX_OK;
  // long segments are rare: handle them one by one from the host copy
  unsigned long long* tmp = nullptr;
  for (int64_t r = 0; r < (int64_t)h_ptr.size() - 1 && rc == SX_OK; ++r) {
    int32_t L = h_ptr[r + 1] - h_ptr[r];
    if (L <= 2048) continue;
    if (!tmp) {
      int32_t maxL = 0;
      for (int64_t q = 0; q < m; ++q) maxL = std::max(maxL, h_ptr[q + 1] - h_ptr[q]);
      rc = dev_alloc((void**)&tmp, (size_t)maxL * 8);
      if (rc) break;
    }
    unsigned long long* seg = keys + h_ptr[r];
    k_sort_chunks<<<(L + 2047) / 2048, kBlock, 0, ctx->stream>>>(seg, L);
    ctx->launches++;
    unsigned long long *src = seg, *dst = tmp;
    for (int32_t w = 2048; w < L; w *= 2) {
      k_merge_pass<<<(L + kBlock - 1) / kBlock, kBlock, 0, ctx->stream>>>(src, dst, L, w);
      ctx->launches++;
      std::swap(src, dst);
    }
    if (src != seg) {
      cudaMemcpyAsync(seg, src, (size_t)L * 8, cudaMemcpyDeviceToDevice, ctx->stream);
    }
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess && rc == SX_OK) rc = cuda_fail(e, "segmented sort", __FILE__, __LINE__);
  dev_free(tmp);
  dev_free(lists);
  dev_free(counts);
  return rc;
}

namespace {

template <typename T>
__global__ void k_gather_sorted(const unsigned long long* __restrict__ keys, int64_t nnz,
                                const T* __restrict__ vals_in, int32_t* indices, T* vals) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += stride) {
    unsigned long long k = keys[p];
    indices[p] = (int32_t)(k >> 32);
    vals[p] = vals_in[(uint32_t)(k & 0xffffffffull)];
  }
}

template <typename T>
__global__ void k_gather_transpose(const unsigned long long* __restrict__ keys, int64_t nnz,
                                   const T* __restrict__ vals_in, int32_t* indices, T* vals) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += stride) {
    unsigned long long k = keys[p];
    if (k == ~0ull) {  // a slot no row range reached keeps (0, 0)
      indices[p] = 0;
      vals[p] = T(0);
    } else {
      indices[p] = (int32_t)(k & 0xffffffffull);
      vals[p] = vals_in[(uint32_t)(k >> 32)];
    }
  }
}

// raw CSR validation (u64 arrays): flags[0] non-monotone, flags[1] some
// index >= ncols, max index, max indptr value; plus narrowing to int32.
__global__ void k_raw_check(const uint64_t* __restrict__ indptr, int64_t plen,
                            const uint64_t* __restrict__ indices, int64_t nnz, uint64_t ncols,
                            int32_t* ptr32, int32_t* idx32, int* flags,
                            unsigned long long* maxes) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t i = tid; i < plen; i += stride) {
    uint64_t v = indptr[i];
    if (i > 0 && v < indptr[i - 1]) flags[0] = 1;
    atomicMax(maxes + 1, (unsigned long long)v);
    ptr32[i] = v > 2147483647ull ? 0 : (int32_t)v;
  }
  for (int64_t k = tid; k < nnz; k += stride) {
    uint64_t c = indices[k];
    if (c >= ncols) flags[1] = 1;
    atomicMax(maxes + 0, (unsigned long long)c);
    idx32[k] = c > 2147483647ull ? 0 : (int32_t)c;
  }
}

__global__ void k_sorted_check(const int32_t* __restrict__ ptr, int64_t nrows,
                               const int32_t* __restrict__ idx, int64_t nnz, int* unsorted) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    int32_t s = ptr[r], e = ptr[r + 1];
    for (int32_t i = s; i + 1 < e; ++i)
      if (i + 1 < nnz && idx[i] > idx[i + 1]) { *unsorted = 1; break; }
  }
}

__global__ void k_row_stats(const int32_t* __restrict__ ptr, int64_t nrows, int* flags,
                            int* maxlen, int* maxchunk) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int mx = 0, mc = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    int32_t L = ptr[r + 1] - ptr[r];
    if (L < 0) flags[0] = 1;
    mx = max(mx, L);
    if ((r & (kBlock - 1)) == 0) {
      const int64_t re = min(nrows, r + kBlock);
      mc = max(mc, ptr[re] - ptr[r]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    mc = max(mc, __shfl_down_sync(0xffffffffu, mc, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(maxlen, mx);
    atomicMax(maxchunk, mc);
  }
}

template <typename TO, typename TI>
__global__ void k_convert(const TI* __restrict__ in, TO* out, int64_t n) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (TO)in[i];
}

__global__ void k_widen_ptr(const int32_t* __restrict__ in, uint64_t* out, int64_t n) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (uint64_t)(uint32_t)in[i];
}
__global__ void k_i64_to_i32(const int64_t* __restrict__ in, int32_t* out, int64_t n, int* bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int64_t v = in[i];
    if (v < 0 || v > 2147483647ll) *bad = 1;
    out[i] = (int32_t)v;
  }
}
__global__ void k_check_cols32(const int32_t* __restrict__ idx, int64_t n, int64_t ncols, int* bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int32_t c = idx[i];
    if (c < 0 || (int64_t)c >= ncols) *bad = 1;
  }
}

}  // namespace

// tile_row[u] = first row r with indptr[r+1] > u * kUnit: the row holding
// entry u * kUnit.  Each nonempty row writes the units that start inside it;
// tile_row[0] = 0 covers leading empty rows and tile_row[units] = nrows.
__global__ void k_tile_rows(const int32_t* __restrict__ ptr, int64_t nrows, int64_t units, int32_t* tr) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    const int64_t lo = ptr[r], hi = ptr[r + 1];
    if (hi <= lo) continue;
    int64_t u = (lo + kUnit - 1) / kUnit;
    if (u == 0) u = 1;
    for (; u * kUnit < hi; ++u) tr[u] = (int32_t)r;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    tr[0] = 0;
    tr[units] = (int32_t)nrows;
  }
}

// smallest and largest column of every 256-row chunk
__global__ void k_chunk_span(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t nrows,
                             int32_t* cmin, int32_t* cmax) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    int32_t lo = INT_MAX, hi = -1;
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) {
      lo = min(lo, idx[k]);
      hi = max(hi, idx[k]);
    }
    if (hi >= 0) {
      atomicMin(cmin + r / kBlock, lo);
      atomicMax(cmax + r / kBlock, hi);
    }
  }
}
// widest chunk span; chunks without entries get base 0
__global__ void k_chunk_base(int32_t* cmin, const int32_t* __restrict__ cmax, int64_t nchunks, int* wide) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += stride) {
    if (cmax[c] < 0) { cmin[c] = 0; continue; }
    if (cmax[c] - cmin[c] > 65535) *wide = 1;
  }
}
__global__ void k_fill_col16(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t nrows,
                             const int32_t* __restrict__ base, uint16_t* col16) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    const int32_t b = base[r / kBlock];
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) col16[k] = (uint16_t)(idx[k] - b);
  }
}

static int csr_prepare_col16(sx_ctx ctx, DevCsr& c) {
  const int64_t nchunks = (c.nrows + kBlock - 1) / kBlock;
  int32_t *cmin = nullptr, *cmax = nullptr;
  int* wide = nullptr;
  uint16_t* col16 = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&cmin, nchunks * 4))) break;
    if ((rc = dev_alloc((void**)&cmax, nchunks * 4))) break;
    if ((rc = dev_alloc((void**)&wide, 4))) break;
    cudaMemsetAsync(cmin, 0x7f, nchunks * 4, ctx->stream);  // 0x7f7f7f7f > any column
    cudaMemsetAsync(cmax, 0xff, nchunks * 4, ctx->stream);  // -1
    cudaMemsetAsync(wide, 0, 4, ctx->stream);
    k_chunk_span<<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(c.indptr, c.indices, c.nrows, cmin, cmax);
    k_chunk_base<<<vec_grid(ctx, nchunks), kBlock, 0, ctx->stream>>>(cmin, cmax, nchunks, wide);
    ctx->launches += 2;
    int h = 1;
    cudaMemcpyAsync(&h, wide, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "column spans", __FILE__, __LINE__); break; }
    if (h) break;  // some chunk spans too many columns: keep the int32 columns only
    if ((rc = dev_alloc((void**)&col16, c.nnz * 2))) break;
    k_fill_col16<<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(c.indptr, c.indices, c.nrows, cmin, col16);
    ctx->launches++;
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "compressed columns", __FILE__, __LINE__); break; }
    c.col16 = col16;
    c.chunk_base = cmin;
    col16 = nullptr;
    cmin = nullptr;
  } while (0);
  dev_free(cmin);
  dev_free(cmax);
  dev_free(wide);
  dev_free(col16);
  return rc;
}

__global__ void k_to_half(const float* __restrict__ in, __half* out, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = __float2half_rn(in[i]);
}

int csr_make_half(sx_ctx ctx, DevCsr& c) {
  dev_free(c.vals16);
  c.vals16 = nullptr;
  dev_free(c.dia_vals16);
  c.dia_vals16 = nullptr;
  if (c.nnz <= 0) return SX_OK;
  SX_CHECK(dev_alloc(&c.vals16, c.nnz * 2));
  k_to_half<<<vec_grid(ctx, c.nnz), kBlock, 0, ctx->stream>>>((const float*)c.vals, (__half*)c.vals16, c.nnz);
  ctx->launches++;
  if (c.dia_vals) {
    const int64_t m = (int64_t)c.dia_n * c.dia_ld;
    SX_CHECK(dev_alloc(&c.dia_vals16, m * 2));
    k_to_half<<<vec_grid(ctx, m), kBlock, 0, ctx->stream>>>((const float*)c.dia_vals, (__half*)c.dia_vals16, m);
    ctx->launches++;
  }
  SX_CUDA(cudaGetLastError());
  return SX_OK;
}

// Sliced layout fill: one warp per slice, lane q copies row q of the slice
// (rows in bin_perm order) to positions sl_base[s] + 32 j + q, zero past the
// row's end (column 0: a valid index, never summed).
template <typename T>
__global__ void k_sliced_fill(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const T* __restrict__ val, const int32_t* __restrict__ perm,
                              const int64_t* __restrict__ base, int64_t nrows, int64_t nslices, int32_t* scols,
                              T* svals) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; s < nslices; s += nwarps) {
    const int64_t B = base[s];
    const int32_t Lg = (int32_t)((base[s + 1] - B) / 32);
    const int64_t p = s * 32 + lane;
    int32_t st = 0, len = 0;
    if (p < nrows) {
      const int32_t r = perm[p];
      st = ptr[r];
      len = ptr[r + 1] - st;
    }
    for (int32_t j = 0; j < Lg; ++j) {
      const bool in = j < len;
      scols[B + (int64_t)j * 32 + lane] = in ? idx[st + j] : 0;
      svals[B + (int64_t)j * 32 + lane] = in ? val[st + j] : T(0);
    }
  }
}

void free_sliced(DevCsr& c) {
  dev_free(c.bin_perm);
  dev_free(c.sl_cols);
  dev_free(c.sl_vals);
  dev_free(c.sl_base);
  dev_free(c.sl_len);
  c.bin_perm = nullptr;
  c.sl_cols = nullptr;
  c.sl_vals = nullptr;
  c.sl_base = nullptr;
  c.sl_len = nullptr;
  c.sl_slices = c.sl_big = c.sl_short = 0;
}

// Rows by length, longest first (a stable counting sort on the host over
// min(length, 4096)), and the sliced layout over that order: slice bases
// and row lengths on the host, the columns and values by k_sliced_fill.
static int csr_prepare_sliced(sx_ctx ctx, DevCsr& c, int w) {
  const int64_t n = c.nrows;
  std::vector<int32_t> ptr(n + 1);
  SX_CUDA(cudaMemcpyAsync(ptr.data(), c.indptr, (n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> start(kBinBuckets + 2, 0);
  auto key = [&](int64_t r) { return (int)std::min<int64_t>(ptr[r + 1] - ptr[r], kBinBuckets); };
  for (int64_t r = 0; r < n; ++r) start[kBinBuckets - key(r) + 1] += 1;  // bucket 0 = longest
  for (int b = 0; b <= kBinBuckets; ++b) start[b + 1] += start[b];
  std::vector<int32_t> perm(std::max<int64_t>(n, 1));
  for (int64_t r = 0; r < n; ++r) perm[start[kBinBuckets - key(r)]++] = (int32_t)r;
  const int64_t ns = (n + 31) / 32;
  std::vector<int32_t> len(ns * 32, 0);
  std::vector<int64_t> base(ns + 1, 0);
  int64_t big = 0, shrt = 0;
  for (int64_t s = 0; s < ns; ++s) {
    int32_t lmax = 0;
    for (int q = 0; q < 32 && s * 32 + q < n; ++q) {
      const int32_t r = perm[s * 32 + q];
      len[s * 32 + q] = ptr[r + 1] - ptr[r];
      lmax = std::max(lmax, len[s * 32 + q]);
    }
    base[s + 1] = base[s] + 32 * (int64_t)lmax;
    // the length order makes both sets prefixes of the slices
    if (lmax > kSlBig) big = s + 1;
    if (lmax > kSlShort) shrt = s + 1;
  }
  const int64_t m = std::max<int64_t>(base[ns], 1);
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&c.bin_perm, std::max<int64_t>(n, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&c.sl_base, (ns + 1) * 8))) break;
    if ((rc = dev_alloc((void**)&c.sl_len, std::max<int64_t>(ns * 32, 1) * 4))) break;
    if ((rc = dev_alloc((void**)&c.sl_cols, m * 4))) break;
    if ((rc = dev_alloc(&c.sl_vals, m * w))) break;
    cudaMemcpyAsync(c.bin_perm, perm.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(c.sl_base, base.data(), (ns + 1) * 8, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(c.sl_len, len.data(), ns * 32 * 4, cudaMemcpyHostToDevice, ctx->stream);
    const int g = (int)std::min<int64_t>((ns + kWarps - 1) / kWarps, (int64_t)ctx->num_sms * 8);
    if (w == 8)
      k_sliced_fill<double><<<g, kBlock, 0, ctx->stream>>>(c.indptr, c.indices, (const double*)c.vals, c.bin_perm,
                                                           c.sl_base, n, ns, c.sl_cols, (double*)c.sl_vals);
    else
      k_sliced_fill<float><<<g, kBlock, 0, ctx->stream>>>(c.indptr, c.indices, (const float*)c.vals, c.bin_perm,
                                                          c.sl_base, n, ns, c.sl_cols, (float*)c.sl_vals);
    ctx->launches++;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "sliced layout", __FILE__, __LINE__);
  } while (0);
  if (rc != SX_OK) {
    free_sliced(c);
    return rc;
  }
  c.sl_slices = ns;
  c.sl_big = big;
  c.sl_short = shrt;
  return SX_OK;
}

int csr_prepare_tiles(sx_ctx ctx, DevCsr& c, int w) {
  dev_free(c.tile_row);
  dev_free(c.col16);
  dev_free(c.chunk_base);
  free_sliced(c);
  c.tile_row = nullptr;
  c.col16 = nullptr;
  c.chunk_base = nullptr;
  c.units = 0;
  if (!c.monotone || c.nnz <= 0 || c.nrows <= 0) return SX_OK;
  // only what this context's kernel choice can use: the 16-bit columns when
  // SX_COL16=1, the unit table when the windowed kernel may run
  if (ctx->col16) SX_CHECK(csr_prepare_col16(ctx, c));
  const bool pipe_fits = c.max_chunk_nnz + 3 <= kBlock * 12;
  if (ctx->win_mode == 0 || (ctx->win_mode == 1 && pipe_fits)) return SX_OK;
  int32_t first = -1;
  SX_CUDA(cudaMemcpyAsync(&first, c.indptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (first != 0) return SX_OK;
  const int64_t units = (c.nnz + kUnit - 1) / kUnit;
  SX_CHECK(dev_alloc((void**)&c.tile_row, (units + 1) * 4));
  k_tile_rows<<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(c.indptr, c.nrows, units, c.tile_row);
  ctx->launches++;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    dev_free(c.tile_row);
    c.tile_row = nullptr;
    return cuda_fail(e, "tile rows", __FILE__, __LINE__);
  }
  c.units = units;
  if (ctx->bin && c.max_row_len > kBinLong && (w == 4 || w == 8)) {
    // the sliced layout is a second copy of the matrix: without the memory
    // for it the windowed kernel serves the matrix instead
    const int rc = csr_prepare_sliced(ctx, c, w);
    if (rc == SX_ERR_OUT_OF_MEMORY) {
      (void)cudaGetLastError();
      return clear_error();
    }
    SX_CHECK(rc);
  }
  return SX_OK;
}

// ---- diagonal layout -------------------------------------------------
// flags[0]: more than kDiaMax distinct offsets; flags[1]: a row whose
// columns do not strictly increase, or a row longer than kDiaMax
__global__ void k_dia_offsets(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                              int* table, int* flags) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int32_t s = ptr[r], e = ptr[r + 1];
    if (e - s > kDiaMax) {
      flags[1] = 1;
      continue;
    }
    int32_t prev = INT_MIN;
    for (int32_t k = s; k < e; ++k) {
      const int32_t c = idx[k];
      if (c <= prev) flags[1] = 1;
      prev = c;
      const int off = c - (int)r;
      bool found = false;
      for (int q = 0; q < kDiaMax && !found; ++q) {
        const int v = table[q];
        if (v == off) {
          found = true;
        } else if (v == INT_MIN) {
          const int old = atomicCAS(table + q, INT_MIN, off);
          found = old == INT_MIN || old == off;
        }
      }
      if (!found) flags[0] = 1;
    }
  }
}

struct DiaTable {
  int32_t off[kDiaMax];
};

template <typename T>
__global__ void k_dia_fill(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const T* __restrict__ val, int64_t n, DiaTable tab, int nd, int64_t ld, T* dv,
                           uint16_t* mask) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    unsigned m = 0;
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) {
      const int off = idx[k] - (int)r;
      int d = 0;
      while (d < nd && tab.off[d] != off) ++d;
      if (d == nd) continue;  // cannot happen once every offset is in the table
      dv[(int64_t)d * ld + r] = val[k];
      m |= 1u << d;
    }
    mask[r] = (uint16_t)m;
  }
}

static void free_dia(DevCsr& c) {
  dev_free(c.dia_vals);
  dev_free(c.dia_vals16);
  dev_free(c.dia_mask);
  c.dia_vals = nullptr;
  c.dia_vals16 = nullptr;
  c.dia_mask = nullptr;
  c.dia_n = 0;
  c.dia_ld = 0;
}

// Builds the diagonal layout when it fits (at most kDiaMax diagonals, rows
// strictly increasing, at most 25 % padding); otherwise leaves none.
int csr_prepare_dia(sx_ctx ctx, DevCsr& c, int w) {
  free_dia(c);
  if (!ctx->dia || w == 0 || !c.monotone || c.nnz <= 0 || c.nrows <= 0 || c.nrows != c.ncols ||
      c.max_row_len > kDiaMax)
    return SX_OK;
  int* d = nullptr;
  SX_CHECK(dev_alloc((void**)&d, (kDiaMax + 2) * sizeof(int)));
  std::vector<int> init(kDiaMax + 2, INT_MIN);
  init[kDiaMax] = init[kDiaMax + 1] = 0;
  SX_CUDA(cudaMemcpyAsync(d, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  k_dia_offsets<<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(c.indptr, c.indices, c.nrows, d, d + kDiaMax);
  ctx->launches++;
  std::vector<int> h(kDiaMax + 2);
  SX_CUDA(cudaMemcpyAsync(h.data(), d, h.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  dev_free(d);
  if (e != cudaSuccess) return cuda_fail(e, "diagonal offsets", __FILE__, __LINE__);
  if (h[kDiaMax] || h[kDiaMax + 1]) return SX_OK;
  std::vector<int32_t> offs;
  for (int q = 0; q < kDiaMax; ++q)
    if (h[q] != INT_MIN) offs.push_back(h[q]);
  std::sort(offs.begin(), offs.end());
  const int nd = (int)offs.size();
  // row stride of the diagonals: a multiple of 32 rows plus an odd number of
  // 32-row groups, so the diagonals (read together) do not start at the same
  // offset of a power-of-two span of memory
  const int64_t ld = (c.nrows + 31) / 32 * 32 + 32 * 37;
  if ((double)nd * (double)c.nrows > 1.25 * (double)c.nnz) return SX_OK;
  if ((int64_t)nd * ld >= ((int64_t)1 << 31)) return SX_OK;  // the kernels index with 32 bits
  DiaTable tab;
  for (int q = 0; q < kDiaMax; ++q) tab.off[q] = q < nd ? offs[q] : 0;
  SX_CHECK(dev_alloc(&c.dia_vals, (size_t)nd * ld * w));
  int rc = dev_alloc((void**)&c.dia_mask, (size_t)c.nrows * 2);
  if (rc != SX_OK) {
    free_dia(c);
    return rc;
  }
  SX_CUDA(cudaMemsetAsync(c.dia_vals, 0, (size_t)nd * ld * w, ctx->stream));
  if (w == 8)
    k_dia_fill<double><<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(
        c.indptr, c.indices, (const double*)c.vals, c.nrows, tab, nd, ld, (double*)c.dia_vals, c.dia_mask);
  else
    k_dia_fill<float><<<vec_grid(ctx, c.nrows), kBlock, 0, ctx->stream>>>(
        c.indptr, c.indices, (const float*)c.vals, c.nrows, tab, nd, ld, (float*)c.dia_vals, c.dia_mask);
  ctx->launches++;
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free_dia(c);
    return cuda_fail(e, "diagonal layout", __FILE__, __LINE__);
  }
  c.dia_n = nd;
  c.dia_ld = ld;
  for (int q = 0; q < kDiaMax; ++q) c.dia_off[q] = tab.off[q];
  return SX_OK;
}

int csr_finalize_stats(sx_ctx ctx, DevCsr& c, int w) {
  int* d = nullptr;
  SX_CHECK(dev_alloc((void**)&d, 4 * sizeof(int)));
  cudaMemsetAsync(d, 0, 4 * sizeof(int), ctx->stream);
  int g = vec_grid(ctx, c.nrows);
  if (c.nrows > 0) {
    k_row_stats<<<g, kBlock, 0, ctx->stream>>>(c.indptr, c.nrows, d, d + 1, d + 3);
    k_sorted_check<<<g, kBlock, 0, ctx->stream>>>(c.indptr, c.nrows, c.indices, c.nnz, d + 2);
    ctx->launches += 2;
  }
  int h[4] = {0, 0, 0, 0};
  cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  dev_free(d);
  if (e != cudaSuccess) return cuda_fail(e, "row stats", __FILE__, __LINE__);
  c.monotone = h[0] == 0;
  c.max_row_len = h[1];
  c.has_sorted_indices = h[2] == 0;
  c.max_chunk_nnz = h[3];
  c.mean_row_len = c.nrows > 0 ? (double)c.nnz / (double)c.nrows : 0.0;
  SX_CHECK(csr_prepare_tiles(ctx, c, w));
  return csr_prepare_dia(ctx, c, w);
}

static std::atomic<uint64_t> g_op_serial{1};

// Every operator gets a serial never used before in this process: the
// solvers' graph caches are keyed by serials, and a key that came back after
// its operator was freed would replay a graph over freed buffers.
uint64_t next_op_serial() { return g_op_serial.fetch_add(1); }

static sx_op new_op(sx_ctx ctx, int kind, int dtype, int64_t nrows, int64_t ncols) {
  sx_op op = new sx_op_s();
  op->kind = kind;
  op->dtype = dtype;
  op->device = ctx->device;
  op->nrows = nrows;
  op->ncols = ncols;
  op->serial = next_op_serial();
  return op;
}

static void free_csr(DevCsr& c) {
  free_dia(c);
  dev_free(c.indptr);
  dev_free(c.indices);
  dev_free(c.vals);
  dev_free(c.tile_row);
  free_sliced(c);
  dev_free(c.col16);
  dev_free(c.chunk_base);
  dev_free(c.vals16);
  c.col16 = nullptr;
  c.chunk_base = nullptr;
  c.vals16 = nullptr;
  c.indptr = nullptr;
  c.indices = nullptr;
  c.vals = nullptr;
  c.tile_row = nullptr;
  c.units = 0;
}

}  // namespace sx

// ============================================================ C ABI
using namespace sx;

namespace sx {
void ic0_destroy(IC0Dev* p);  // sx_ic0.cu
void destroy_op_internal(sx_op op) {
  if (!op) return;
  free_csr(op->csr);
  dev_free(op->diag);
  dev_free(op->work);
  if (op->transpose) destroy_op_internal(op->transpose);
  if (op->sym_low) destroy_op_internal(op->sym_low);
  if (op->ic0) ic0_destroy(op->ic0);
  if (op->tri) tri_destroy(op->tri);
  delete op;
}
}  // namespace sx

extern "C" {

void sx_last_error(sx_error_info* out) {
  if (out) *out = g_err;
}

const char* sx_status_string(int s) {
  switch (s) {
    case SX_OK: return "ok";
    case SX_ERR_COMPUTATION: return "ComputationError";
    case SX_ERR_DIMENSION_MISMATCH: return "DimensionMismatch";
    case SX_ERR_INDEX_OUT_OF_BOUNDS: return "IndexOutOfBounds";
    case SX_ERR_INVALID_AXIS: return "InvalidAxis";
    case SX_ERR_INVALID_SLICE_RANGE: return "InvalidSliceRange";
    case SX_ERR_INCONSISTENT_DATA: return "InconsistentData";
    case SX_ERR_NOT_IMPLEMENTED: return "NotImplemented";
    case SX_ERR_SINGULAR_MATRIX: return "SingularMatrix";
    case SX_ERR_VALUE: return "ValueError";
    case SX_ERR_CONVERSION: return "ConversionError";
    case SX_ERR_OPERATION_NOT_SUPPORTED: return "OperationNotSupported";
    case SX_ERR_SHAPE_MISMATCH: return "ShapeMismatch";
    case SX_ERR_ITERATIVE_SOLVER_FAILURE: return "IterativeSolverFailure";
    case SX_ERR_INDEX_CAST_OVERFLOW: return "IndexCastOverflow";
    case SX_ERR_CUDA: return "CudaError";
    case SX_ERR_DEVICE_TIMEOUT: return "DeviceTimeout";
    case SX_ERR_INVALID_ARGUMENT: return "InvalidArgument";
    case SX_ERR_OUT_OF_MEMORY: return "OutOfMemory";
    default: return "unknown";
  }
}

const char* sx_message_string(int m) {
  switch (m) {
    case MSG_CONVERGED: return "Converged";
    case MSG_MAX_ITER: return "Maximum iterations reached";
    case MSG_NOT_PD: return "Matrix not positive definite (p^T*A*p <= 0)";
    case MSG_CONVERGED_INITIAL: return "Converged with initial guess";
    case MSG_BD_RHO: return "BiCGSTAB breakdown: rho \xE2\x89\x88 0";
    case MSG_BD_RHAT_V: return "BiCGSTAB breakdown: (r_hat, v) \xE2\x89\x88 0";
    case MSG_BD_ALPHA: return "BiCGSTAB breakdown: alpha is not finite";
    case MSG_BD_TT: return "BiCGSTAB breakdown: (t, t) \xE2\x89\x88 0";
    case MSG_BD_OMEGA: return "BiCGSTAB breakdown: omega is not finite or too small";
    case MSG_BICG_PQ: return "BiCG breakdown: (p_star, q) \xE2\x89\x88 0";
    case MSG_BICG_RHO: return "BiCG breakdown: rho \xE2\x89\x88 0";
    case MSG_CGS_RHO: return "CGS breakdown: rho \xE2\x89\x88 0";
    case MSG_CGS_SIGMA: return "CGS breakdown: sigma \xE2\x89\x88 0";
    case MSG_QMR_INITIAL: return "Converged at initial guess";
    case MSG_QMR_RHO: return "Breakdown: rho = 0";
    case MSG_QMR_PQ: return "Breakdown: <p_tilde, q> = 0";
    case MSG_QMR_CONVERGED: return "Converged in {iterations} iterations";
    case MSG_QMR_OMEGA: return "Breakdown: omega = 0";
    case MSG_QMR_MAX_ITER: return "Did not converge in {max_iter} iterations. Residual: {r}";
    case MSG_ZERO_RHS: return "System has zero right-hand side";
    case MSG_ZERO_RESIDUAL: return "Initial residual is zero";
    default: return "";
  }
}

static int ctx_init(int device, cudaStream_t stream, bool own, sx_ctx* out) {
  if (!out) return err_arg("out is null");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(device));
  int sms = 0;
  SX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  sx_ctx c = new sx_ctx_s();
  c->device = device;
  c->num_sms = sms;
  c->own_stream = own;
  if (const char* t = std::getenv("SX_WIN")) c->win_mode = std::atoi(t);
  if (const char* t = std::getenv("SX_DIA")) c->dia = std::atoi(t);
  if (const char* t = std::getenv("SX_DIA_ND6")) c->dia_nd6 = std::strcmp(t, "0") != 0;
  if (const char* t = std::getenv("SX_DIA_BAND")) c->dia_band = std::strcmp(t, "0") != 0;
  if (const char* t = std::getenv("SX_PDL")) c->pdl = std::strcmp(t, "0") != 0;
  if (const char* t = std::getenv("SX_BIN")) c->bin = std::strcmp(t, "0") != 0;
  if (const char* t = std::getenv("SX_COL16")) c->col16 = std::strcmp(t, "1") == 0;
  if (const char* t = std::getenv("SX_MX_FUSED")) c->mx_unfused = std::strcmp(t, "0") == 0;
  if (const char* t = std::getenv("SX_SHORT")) c->short_rows = std::atoi(t);
  if (const char* t = std::getenv("SX_WIN_SHAPE")) c->win_shape = std::atoi(t);
  if (own) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
    }
  } else {
    c->stream = stream;
  }
  mem_cache_register_stream(device, c->stream);
  *out = c;
  return clear_error();
}

int sx_ctx_create(int device, sx_ctx* out) { return ctx_init(device, nullptr, true, out); }
int sx_ctx_create_on_stream(int device, void* stream, sx_ctx* out) {
  return ctx_init(device, (cudaStream_t)stream, false, out);
}

void sx_solver_cache_release(sx_ctx ctx);  // sx_krylov.cu

int sx_ctx_destroy(sx_ctx ctx) {
  if (!ctx) return SX_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  sx_solver_cache_release(ctx);
  dev_free(ctx->red_partials);
  dev_free(ctx->red_counter);
  dev_free(ctx->scratch);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  mem_cache_unregister_stream(ctx->device, ctx->stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SX_OK;
}

int sx_mem_cache_trim(void) {
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lk(bc.mu);
  int cur = 0;
  cudaGetDevice(&cur);
  std::vector<int> devs;
  for (const auto& h : bc.held) devs.push_back(h.first);
  for (int d : devs) {
    cudaSetDevice(d);
    cache_release_device(bc, d);
  }
  cudaSetDevice(cur);
  return SX_OK;
}

uint64_t sx_mem_cache_bytes(void) {
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lk(bc.mu);
  uint64_t t = 0;
  for (const auto& h : bc.held) t += h.second;
  return t;
}
void* sx_ctx_stream(sx_ctx ctx) { return ctx ? (void*)ctx->stream : nullptr; }
int sx_ctx_synchronize(sx_ctx ctx) {
  if (!ctx) return err_arg("ctx is null");
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  return SX_OK;
}
uint64_t sx_ctx_kernel_launches(sx_ctx ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------- triplets
int sx_csr_from_triplets(sx_ctx ctx, sx_dtype dtype, sx_csr_api api, const uint64_t* rows,
                         const uint64_t* cols, const void* data, uint64_t nnz, uint64_t nrows,
                         uint64_t ncols, int sorted, sx_op* out) {
  if (!ctx || !out) return err_arg("null ctx/out");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  if (nnz > 0 && (!rows || !cols || !data)) return err_arg("null triplet arrays");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  const size_t w = elt_size(dtype);
  if (nnz > kI32Max) return err_cast(nnz);
  // device copies of the triplets
  uint64_t *d_rows = nullptr, *d_cols = nullptr;
  int32_t *rows32 = nullptr, *cols32 = nullptr, *cnt = nullptr, *cursor = nullptr;
  void* d_data = nullptr;
  int* flags = nullptr;
  unsigned long long *first_bad = nullptr, *keys = nullptr;
  DevCsr c;
  int rc = SX_OK;
  auto cleanup = [&]() {
    dev_free(d_rows); dev_free(d_cols); dev_free(rows32); dev_free(cols32); dev_free(cnt);
    dev_free(cursor); dev_free(d_data); dev_free(flags); dev_free(first_bad); dev_free(keys);
  };
  const int64_t n = (int64_t)nnz;
  do {
    if (n > 0) {
      if ((rc = dev_alloc((void**)&d_rows, n * 8))) break;
      if ((rc = dev_alloc((void**)&d_cols, n * 8))) break;
      if ((rc = dev_alloc((void**)&rows32, n * 4))) break;
      if ((rc = dev_alloc((void**)&cols32, n * 4))) break;
      if ((rc = dev_alloc(&d_data, n * w))) break;
    }
    if ((rc = dev_alloc((void**)&flags, 4 * sizeof(int)))) break;
    if ((rc = dev_alloc((void**)&first_bad, 8))) break;
    cudaMemsetAsync(flags, 0, 4 * sizeof(int), ctx->stream);
    cudaMemsetAsync(first_bad, 0xff, 8, ctx->stream);
    if (n > 0) {
      cudaMemcpyAsync(d_rows, rows, n * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(d_cols, cols, n * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(d_data, data, n * w, cudaMemcpyHostToDevice, ctx->stream);
      k_triplet_check<<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
          d_rows, d_cols, n, nrows, ncols, rows32, cols32, flags, first_bad);
      ctx->launches++;
    }
    int hf[4];
    unsigned long long hb = 0;
    cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&hb, first_bad, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "triplet upload", __FILE__, __LINE__); break; }
    if (api == SX_API_CSR_MATRIX) {
      // csr.rs:107-119: rows first, then columns
      if (hf[0]) { rc = err_value("Row index out of bounds"); break; }
      if (hf[1]) { rc = err_value("Column index out of bounds"); break; }
    } else {
      // csr_array.rs:178-186: the first offending triplet in input order
      if (n > 0 && (hf[0] || hf[1])) {
        uint64_t r = 0, cc = 0;
        cudaMemcpy(&r, d_rows + hb, 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(&cc, d_cols + hb, 8, cudaMemcpyDeviceToHost);
        rc = err_oob(r, cc, nrows, ncols);
        break;
      }
    }
    if (nrows > kI32Max - 1 || ncols > kI32Max) {
      // the first row index, then the first column index, that does not fit;
      // else the dimension itself
      uint64_t v = first_cast_overflow(rows, nnz);
      if (!v) v = first_cast_overflow(cols, nnz);
      rc = err_cast(v ? v : (nrows > kI32Max - 1 ? nrows : ncols));
      break;
    }
    c.nrows = (int64_t)nrows;
    c.ncols = (int64_t)ncols;
    c.nnz = n;
    if ((rc = dev_alloc((void**)&c.indptr, (nrows + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&c.indices, n * 4))) break;
    if ((rc = dev_alloc(&c.vals, n * w))) break;
    if ((rc = dev_alloc((void**)&cnt, (nrows + 1) * 4))) break;
    cudaMemsetAsync(cnt, 0, (nrows + 1) * 4, ctx->stream);
    if (n > 0) {
      k_count<<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(rows32, n, cnt);
      ctx->launches++;
    }
    if ((rc = scan_exclusive(ctx, cnt, (int64_t)nrows, c.indptr))) break;
    const bool do_sort = (api == SX_API_CSR_MATRIX) || !sorted;
    if (n > 0 && do_sort) {
      if ((rc = dev_alloc((void**)&cursor, (nrows + 1) * 4))) break;
      if ((rc = dev_alloc((void**)&keys, n * 8))) break;
      cudaMemsetAsync(cursor, 0, (nrows + 1) * 4, ctx->stream);
      k_scatter_rows<<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(rows32, cols32, n, c.indptr,
                                                                      cursor, keys);
      ctx->launches++;
      std::vector<int32_t> hptr;
      if ((rc = long_segment_ptr(ctx, cnt, (int64_t)nrows, c.indptr, hptr))) break;
      if ((rc = segmented_sort(ctx, c.indptr, (int64_t)nrows, keys, hptr))) break;
      if (dtype == SX_F64)
        k_gather_sorted<double><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            keys, n, (const double*)d_data, c.indices, (double*)c.vals);
      else
        k_gather_sorted<float><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            keys, n, (const float*)d_data, c.indices, (float*)c.vals);
      ctx->launches++;
    } else if (n > 0) {
      // sorted=true: the triplets are taken in input order (csr_array.rs:192-214)
      cudaMemcpyAsync(c.indices, cols32, n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaMemcpyAsync(c.vals, d_data, n * w, cudaMemcpyDeviceToDevice, ctx->stream);
    }
    if ((rc = csr_finalize_stats(ctx, c, (int)elt_size(dtype)))) break;
  } while (0);
  cleanup();
  if (rc != SX_OK) {
    free_csr(c);
    return rc;
  }
  sx_op op = new_op(ctx, SX_OP_CSR, dtype, (int64_t)nrows, (int64_t)ncols);
  op->csr = c;
  *out = op;
  return clear_error();
}

// ------------------------------------------------------------------- raw
int sx_csr_from_raw(sx_ctx ctx, sx_dtype dtype, sx_csr_api api, const uint64_t* indptr,
                    uint64_t indptr_len, const uint64_t* indices, const void* data, uint64_t nnz,
                    uint64_t nrows, uint64_t ncols, sx_op* out) {
  if (!ctx || !out) return err_arg("null ctx/out");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  const size_t w = elt_size(dtype);
  if (api == SX_API_CSR_MATRIX) {
    if (indptr_len != nrows + 1) return err_dim(nrows + 1, indptr_len);
  } else {
    if (indptr_len != nrows + 1)
      return err_incons("indptr length (" + std::to_string(indptr_len) +
                        ") must be one more than the number of rows (" + std::to_string(nrows) +
                        ")");
  }
  if (indptr_len > 0 && !indptr) return err_arg("null indptr");
  if (nnz > 0 && (!indices || !data)) return err_arg("null arrays");
  if (nnz > kI32Max) return err_cast(nnz);
  if (nrows > kI32Max - 1) return err_cast(nrows);
  const int64_t n = (int64_t)nnz, pl = (int64_t)indptr_len;
  uint64_t *d_ptr = nullptr, *d_idx = nullptr;
  int* flags = nullptr;
  unsigned long long* maxes = nullptr;
  DevCsr c;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&d_ptr, pl * 8))) break;
    if ((rc = dev_alloc((void**)&d_idx, std::max<int64_t>(n, 1) * 8))) break;
    if ((rc = dev_alloc((void**)&flags, 4 * sizeof(int)))) break;
    if ((rc = dev_alloc((void**)&maxes, 2 * 8))) break;
    if ((rc = dev_alloc((void**)&c.indptr, pl * 4))) break;
    if ((rc = dev_alloc((void**)&c.indices, std::max<int64_t>(n, 1) * 4))) break;
    if ((rc = dev_alloc(&c.vals, std::max<int64_t>(n, 1) * w))) break;
    cudaMemsetAsync(flags, 0, 4 * sizeof(int), ctx->stream);
    cudaMemsetAsync(maxes, 0, 16, ctx->stream);
    cudaMemcpyAsync(d_ptr, indptr, pl * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (n > 0) {
      cudaMemcpyAsync(d_idx, indices, n * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(c.vals, data, n * w, cudaMemcpyHostToDevice, ctx->stream);
    }
    k_raw_check<<<vec_grid(ctx, std::max(pl, n)), kBlock, 0, ctx->stream>>>(
        d_ptr, pl, d_idx, n, ncols, c.indptr, c.indices, flags, maxes);
    ctx->launches++;
    int hf[4];
    unsigned long long hm[2];
    uint64_t first = 0, last = 0;
    cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(hm, maxes, sizeof(hm), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "raw upload", __FILE__, __LINE__); break; }
    first = indptr[0];
    last = indptr[pl - 1];
    if (api == SX_API_CSR_MATRIX) {
      // csr.rs:182-217 in order
      if (hf[0]) { rc = err_value("Row pointer array must be monotonically increasing"); break; }
      if (last != nnz) { rc = err_value("Last row pointer entry must match data length"); break; }
      if (hf[1]) { rc = err_value("Column index out of bounds"); break; }
    } else {
      // csr_array.rs:98-128 in order
      if (n > 0 && hm[0] >= ncols) { rc = err_oob(0, hm[0], nrows, ncols); break; }
      if (first != 0) { rc = err_incons("first element of indptr must be 0"); break; }
      if (last != nnz) {
        rc = err_incons("last element of indptr (" + std::to_string(last) +
                        ") must equal data length (" + std::to_string(nnz) + ")");
        break;
      }
      // CsrArray::new accepts a decreasing indptr; an entry above the data
      // length would make a row run past the arrays (a slice panic in the
      // reference at first use), so it is refused here
      if (hm[1] > nnz) {
        rc = err_incons("indptr entry (" + std::to_string(hm[1]) + ") exceeds data length (" +
                        std::to_string(nnz) + ")");
        break;
      }
    }
    if (hm[1] > kI32Max) { rc = err_cast(hm[1]); break; }
    if (ncols > kI32Max) {
      const uint64_t v = first_cast_overflow(indices, nnz);
      rc = err_cast(v ? v : ncols);
      break;
    }
    c.nrows = (int64_t)nrows;
    c.ncols = (int64_t)ncols;
    c.nnz = n;
    if ((rc = csr_finalize_stats(ctx, c, (int)w))) break;
  } while (0);
  dev_free(d_ptr); dev_free(d_idx); dev_free(flags); dev_free(maxes);
  if (rc != SX_OK) {
    free_csr(c);
    return rc;
  }
  sx_op op = new_op(ctx, SX_OP_CSR, dtype, (int64_t)nrows, (int64_t)ncols);
  op->csr = c;
  *out = op;
  return clear_error();
}

int sx_csr_from_raw_i32(sx_ctx ctx, sx_dtype dtype, const int64_t* indptr, const int32_t* indices,
                        const void* data, uint64_t nrows, uint64_t ncols, uint64_t nnz, sx_mem mem,
                        sx_op* out) {
  if (!ctx || !out || !indptr) return err_arg("null ctx/out/indptr");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  if (nnz > 0 && (!indices || !data)) return err_arg("null arrays");
  *out = nullptr;
  SX_CUDA(cudaSetDevice(ctx->device));
  if (nnz > kI32Max) return err_cast(nnz);
  if (nrows > kI32Max - 1) return err_cast(nrows);
  if (ncols > kI32Max) return err_cast(ncols);
  const size_t w = elt_size(dtype);
  const int64_t n = (int64_t)nnz, m = (int64_t)nrows;
  const cudaMemcpyKind kind = mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  DevCsr c;
  int64_t* d_ptr64 = nullptr;
  int* bad = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&d_ptr64, (m + 1) * 8))) break;
    if ((rc = dev_alloc((void**)&bad, 16))) break;
    if ((rc = dev_alloc((void**)&c.indptr, (m + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&c.indices, std::max<int64_t>(n, 1) * 4))) break;
    if ((rc = dev_alloc(&c.vals, std::max<int64_t>(n, 1) * w))) break;
    cudaMemsetAsync(bad, 0, 16, ctx->stream);
    cudaMemcpyAsync(d_ptr64, indptr, (m + 1) * 8, kind, ctx->stream);
    if (n > 0) {
      cudaMemcpyAsync(c.indices, indices, n * 4, kind, ctx->stream);
      cudaMemcpyAsync(c.vals, data, n * w, kind, ctx->stream);
    }
    k_i64_to_i32<<<vec_grid(ctx, m + 1), kBlock, 0, ctx->stream>>>(d_ptr64, c.indptr, m + 1, bad);
    if (n > 0)
      k_check_cols32<<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(c.indices, n, (int64_t)ncols,
                                                                     bad + 1);
    ctx->launches += 2;
    int hb[4] = {0, 0, 0, 0};
    int64_t first = 0, last = 0;
    cudaMemcpyAsync(hb, bad, 16, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&first, d_ptr64, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&last, d_ptr64 + m, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "upload", __FILE__, __LINE__); break; }
    if (hb[0]) { rc = err_cast((uint64_t)last); break; }
    if (last != n) { rc = err_value("Last row pointer entry must match data length"); break; }
    if (hb[1]) { rc = err_value("Column index out of bounds"); break; }
    c.nrows = m;
    c.ncols = (int64_t)ncols;
    c.nnz = n;
    if ((rc = csr_finalize_stats(ctx, c, (int)w))) break;
    if (!c.monotone) { rc = err_value("Row pointer array must be monotonically increasing"); break; }
  } while (0);
  dev_free(d_ptr64);
  dev_free(bad);
  if (rc != SX_OK) {
    free_csr(c);
    return rc;
  }
  sx_op op = new_op(ctx, SX_OP_CSR, dtype, m, (int64_t)ncols);
  op->csr = c;
  *out = op;
  return clear_error();
}

}  // extern "C"

// ------------------------------------------------------------- transpose
// stats = false: the arrays only (no row statistics, tiles or diagonal
// layout), for transposes used as index maps
static int csr_transpose_dev(sx_ctx ctx, const DevCsr& a, int dtype, DevCsr& t, bool stats = true) {
  if (!a.monotone)
    return err_incons("transpose needs non-decreasing row pointers");
  const int64_t n = a.nnz;
  const int64_t m = a.ncols;
  int32_t *cnt = nullptr, *cursor = nullptr;
  unsigned long long* keys = nullptr;
  int rc = SX_OK;
  t.nrows = a.ncols;
  t.ncols = a.nrows;
  t.nnz = n;
  do {
    if ((rc = dev_alloc((void**)&t.indptr, (m + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&t.indices, std::max<int64_t>(n, 1) * 4))) break;
    if ((rc = dev_alloc(&t.vals, std::max<int64_t>(n, 1) * elt_size(dtype)))) break;
    if ((rc = dev_alloc((void**)&cnt, (m + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&cursor, (m + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&keys, std::max<int64_t>(n, 1) * 8))) break;
    cudaMemsetAsync(cnt, 0, (m + 1) * 4, ctx->stream);
    cudaMemsetAsync(cursor, 0, (m + 1) * 4, ctx->stream);
    cudaMemsetAsync(keys, 0xff, std::max<int64_t>(n, 1) * 8, ctx->stream);
    // column counts over the whole indices array, as csr.rs:291-294 does
    if (n > 0) {
      k_count<<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(a.indices, n, cnt);
      ctx->launches++;
    }
    if ((rc = scan_exclusive(ctx, cnt, m, t.indptr))) break;
    if (a.nrows > 0 && n > 0) {
      k_scatter_cols<<<vec_grid(ctx, a.nrows), kBlock, 0, ctx->stream>>>(
          a.indptr, a.indices, a.nrows, t.indptr, cursor, keys);
      ctx->launches++;
    }
    std::vector<int32_t> hptr;
    if ((rc = long_segment_ptr(ctx, cnt, m, t.indptr, hptr))) break;
    if ((rc = segmented_sort(ctx, t.indptr, m, keys, hptr))) break;
    if (n > 0) {
      if (dtype == SX_F64)
        k_gather_transpose<double><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            keys, n, (const double*)a.vals, t.indices, (double*)t.vals);
      else
        k_gather_transpose<float><<<vec_grid(ctx, n), kBlock, 0, ctx->stream>>>(
            keys, n, (const float*)a.vals, t.indices, (float*)t.vals);
      ctx->launches++;
    }
    if (stats) {
      rc = csr_finalize_stats(ctx, t, (int)elt_size(dtype));
    } else {
      t.monotone = true;
      t.has_sorted_indices = true;
      t.max_chunk_nnz = std::numeric_limits<int32_t>::max();  // no register-pipeline SpMV
      const cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "transpose", __FILE__, __LINE__);
    }
  } while (0);
  dev_free(cnt);
  dev_free(cursor);
  dev_free(keys);
  if (rc != SX_OK) free_csr(t);
  return rc;
}

namespace sx {
int csr_transpose_internal(sx_ctx ctx, sx_op a, sx_op* out, bool stats) {
  DevCsr t;
  SX_CHECK(csr_transpose_dev(ctx, a->csr, a->dtype, t, stats));
  sx_op op = new_op(ctx, SX_OP_CSR, a->dtype, a->ncols, a->nrows);
  op->csr = t;
  *out = op;
  return SX_OK;
}
sx_op csr_op_adopt(sx_ctx ctx, int dtype, DevCsr& c) {
  sx_op op = new_op(ctx, SX_OP_CSR, dtype, c.nrows, c.ncols);
  op->csr = c;
  c = DevCsr();
  return op;
}
int ensure_transpose(sx_ctx ctx, sx_op a) {
  if (a->transpose) return SX_OK;
  return csr_transpose_internal(ctx, a, &a->transpose);
}
}  // namespace sx

extern "C" {

int sx_csr_transpose(sx_ctx ctx, sx_op a, sx_op* out) {
  if (!ctx || !a || !out) return err_arg("null argument");
  if (a->kind != SX_OP_CSR) return err_arg("not a CSR operator");
  SX_CUDA(cudaSetDevice(ctx->device));
  SX_CHECK(csr_transpose_internal(ctx, a, out));
  return clear_error();
}

int sx_csr_astype(sx_ctx ctx, sx_op a, sx_dtype dtype, sx_op* out) {
  if (!ctx || !a || !out) return err_arg("null argument");
  if (a->kind != SX_OP_CSR) return err_arg("not a CSR operator");
  SX_CUDA(cudaSetDevice(ctx->device));
  DevCsr c = a->csr;
  c.indptr = nullptr; c.indices = nullptr; c.vals = nullptr; c.tile_row = nullptr; c.units = 0;
  c.bin_perm = nullptr; c.sl_cols = nullptr; c.sl_vals = nullptr; c.sl_base = nullptr; c.sl_len = nullptr;
  c.sl_slices = c.sl_big = c.sl_short = 0;
  c.col16 = nullptr; c.chunk_base = nullptr; c.vals16 = nullptr;
  c.dia_vals = nullptr; c.dia_vals16 = nullptr; c.dia_mask = nullptr;
  const int64_t n = a->csr.nnz;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&c.indptr, (c.nrows + 1) * 4))) break;
    if ((rc = dev_alloc((void**)&c.indices, std::max<int64_t>(n, 1) * 4))) break;
    if ((rc = dev_alloc(&c.vals, std::max<int64_t>(n, 1) * elt_size(dtype)))) break;
    cudaMemcpyAsync(c.indptr, a->csr.indptr, (c.nrows + 1) * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    if (n > 0) {
      cudaMemcpyAsync(c.indices, a->csr.indices, n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      int g = vec_grid(ctx, n);
      if (a->dtype == dtype) {
        cudaMemcpyAsync(c.vals, a->csr.vals, n * elt_size(dtype), cudaMemcpyDeviceToDevice, ctx->stream);
      } else if (dtype == SX_F32) {
        k_convert<float, double><<<g, kBlock, 0, ctx->stream>>>((const double*)a->csr.vals, (float*)c.vals, n);
        ctx->launches++;
      } else {
        k_convert<double, float><<<g, kBlock, 0, ctx->stream>>>((const float*)a->csr.vals, (double*)c.vals, n);
        ctx->launches++;
      }
    }
    // the diagonal layout converts along (same positions, new value type)
    if (a->csr.dia_vals && ctx->dia) {
      const int64_t m = (int64_t)c.dia_n * c.dia_ld;
      if ((rc = dev_alloc(&c.dia_vals, m * elt_size(dtype)))) break;
      if ((rc = dev_alloc((void**)&c.dia_mask, c.nrows * 2))) break;
      cudaMemcpyAsync(c.dia_mask, a->csr.dia_mask, c.nrows * 2, cudaMemcpyDeviceToDevice, ctx->stream);
      const int g = vec_grid(ctx, m);
      if (a->dtype == dtype) {
        cudaMemcpyAsync(c.dia_vals, a->csr.dia_vals, m * elt_size(dtype), cudaMemcpyDeviceToDevice, ctx->stream);
      } else if (dtype == SX_F32) {
        k_convert<float, double><<<g, kBlock, 0, ctx->stream>>>((const double*)a->csr.dia_vals, (float*)c.dia_vals, m);
        ctx->launches++;
      } else {
        k_convert<double, float><<<g, kBlock, 0, ctx->stream>>>((const float*)a->csr.dia_vals, (double*)c.dia_vals, m);
        ctx->launches++;
      }
    } else {
      c.dia_n = 0;
      c.dia_ld = 0;
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "astype", __FILE__, __LINE__); break; }
    rc = csr_prepare_tiles(ctx, c, (int)elt_size(dtype));
  } while (0);
  if (rc != SX_OK) { free_csr(c); return rc; }
  sx_op op = new_op(ctx, SX_OP_CSR, dtype, a->nrows, a->ncols);
  op->csr = c;
  *out = op;
  return clear_error();
}

int sx_csr_info(sx_op a, uint64_t* nrows, uint64_t* ncols, uint64_t* nnz, int* has_sorted) {
  if (!a) return err_arg("null op");
  if (a->kind != SX_OP_CSR && a->kind != SX_OP_FSAI) return err_arg("not a CSR operator");
  if (nrows) *nrows = (uint64_t)a->csr.nrows;
  if (ncols) *ncols = (uint64_t)a->csr.ncols;
  if (nnz) *nnz = (uint64_t)a->csr.nnz;
  if (has_sorted) *has_sorted = a->csr.has_sorted_indices ? 1 : 0;
  return SX_OK;
}

int sx_csr_download(sx_ctx ctx, sx_op a, uint64_t* indptr, uint64_t* indices, void* data) {
  if (!ctx || !a) return err_arg("null argument");
  if (a->kind != SX_OP_CSR) return err_arg("not a CSR operator");
  SX_CUDA(cudaSetDevice(ctx->device));
  const DevCsr& c = a->csr;
  uint64_t* tmp = nullptr;
  int64_t big = std::max<int64_t>(c.nrows + 1, c.nnz);
  SX_CHECK(dev_alloc((void**)&tmp, std::max<int64_t>(big, 1) * 8));
  int g = vec_grid(ctx, big);
  if (indptr) {
    k_widen_ptr<<<g, kBlock, 0, ctx->stream>>>(c.indptr, tmp, c.nrows + 1);
    cudaMemcpyAsync(indptr, tmp, (c.nrows + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
  }
  if (indices && c.nnz > 0) {
    k_widen_ptr<<<g, kBlock, 0, ctx->stream>>>(c.indices, tmp, c.nnz);
    cudaMemcpyAsync(indices, tmp, c.nnz * 8, cudaMemcpyDeviceToHost, ctx->stream);
  }
  if (data && c.nnz > 0)
    cudaMemcpyAsync(data, c.vals, c.nnz * elt_size(a->dtype), cudaMemcpyDeviceToHost, ctx->stream);
  ctx->launches += 2;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  dev_free(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "download", __FILE__, __LINE__);
  return clear_error();
}

}  // extern "C"

namespace sx {
namespace {
template <typename T>
__global__ void k_get(const int32_t* ptr, const int32_t* idx, const T* vals, int64_t i, int64_t j,
                      T* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    T v = T(0);
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
      if (idx[k] == (int32_t)j) { v = vals[k]; break; }
    *out = v;
  }
}
}  // namespace
}  // namespace sx

extern "C" {

int sx_csr_get(sx_ctx ctx, sx_op a, uint64_t i, uint64_t j, void* out) {
  if (!ctx || !a || !out) return err_arg("null argument");
  // a symmetric operator's merged rows give SymCsrMatrix::get's first match
  if (a->kind != SX_OP_CSR && a->kind != SX_OP_SYM_CSR) return err_arg("not a CSR operator");
  const size_t w = elt_size(a->dtype);
  // csr.rs:35-37: out-of-range positions read as zero
  if (i >= (uint64_t)a->csr.nrows || j >= (uint64_t)a->csr.ncols) {
    std::memset(out, 0, w);
    return SX_OK;
  }
  void* d = nullptr;
  SX_CHECK(ctx_pinned(ctx, 16, &d));
  void* dv = nullptr;
  SX_CHECK(dev_alloc(&dv, 16));
  if (a->dtype == SX_F64)
    k_get<double><<<1, 32, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const double*)a->csr.vals,
                                           (int64_t)i, (int64_t)j, (double*)dv);
  else
    k_get<float><<<1, 32, 0, ctx->stream>>>(a->csr.indptr, a->csr.indices, (const float*)a->csr.vals,
                                          (int64_t)i, (int64_t)j, (float*)dv);
  ctx->launches++;
  cudaMemcpyAsync(d, dv, w, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  dev_free(dv);
  if (e != cudaSuccess) return cuda_fail(e, "get", __FILE__, __LINE__);
  std::memcpy(out, d, w);
  return SX_OK;
}

// ------------------------------------------------------- simple operators
static int make_vec_op(sx_ctx ctx, int kind, sx_dtype dtype, const void* diag, uint64_t n,
                       sx_op* out) {
  if (!ctx || !out) return err_arg("null argument");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  if (n > kI32Max) return err_cast(n);
  SX_CUDA(cudaSetDevice(ctx->device));
  sx_op op = new_op(ctx, kind, dtype, (int64_t)n, (int64_t)n);
  if (diag) {
    int rc = dev_alloc(&op->diag, std::max<uint64_t>(n, 1) * elt_size(dtype));
    if (rc) { delete op; return rc; }
    cudaMemcpyAsync(op->diag, diag, n * elt_size(dtype), cudaMemcpyHostToDevice, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { destroy_op_internal(op); return cuda_fail(e, "diag upload", __FILE__, __LINE__); }
  }
  *out = op;
  return clear_error();
}

int sx_op_identity(sx_ctx ctx, sx_dtype dtype, uint64_t n, sx_op* out) {
  return make_vec_op(ctx, SX_OP_IDENTITY, dtype, nullptr, n, out);
}
int sx_op_scaled_identity(sx_ctx ctx, sx_dtype dtype, uint64_t n, double scale, sx_op* out) {
  int rc = make_vec_op(ctx, SX_OP_SCALED_IDENTITY, dtype, nullptr, n, out);
  if (rc == SX_OK) (*out)->scale = scale;
  return rc;
}
int sx_op_diagonal(sx_ctx ctx, sx_dtype dtype, const void* diag, uint64_t n, sx_op* out) {
  if (n > 0 && !diag) return err_arg("null diagonal");
  return make_vec_op(ctx, SX_OP_DIAGONAL, dtype, n > 0 ? diag : nullptr, n, out);
}
int sx_op_host(sx_ctx ctx, sx_dtype dtype, uint64_t nrows, uint64_t ncols, sx_host_matvec_fn fn,
               void* user, sx_op* out) {
  if (!ctx || !out || !fn) return err_arg("null argument");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  sx_op op = new_op(ctx, SX_OP_HOST, dtype, (int64_t)nrows, (int64_t)ncols);
  op->host.fn = fn;
  op->host.user = user;
  *out = op;
  return clear_error();
}

int sx_op_zero(sx_ctx ctx, sx_dtype dtype, uint64_t nrows, uint64_t ncols, sx_op* out) {
  if (!ctx || !out) return err_arg("null argument");
  if (dtype != SX_F32 && dtype != SX_F64) return err_arg("dtype");
  if (nrows > kI32Max) return err_cast(nrows);
  if (ncols > kI32Max) return err_cast(ncols);
  *out = new_op(ctx, SX_OP_ZERO, dtype, (int64_t)nrows, (int64_t)ncols);
  return clear_error();
}

static int make_pair_op(sx_ctx ctx, int kind, sx_op a, sx_op b, int64_t nrows, int64_t ncols,
                        int64_t work_len, sx_op* out) {
  if (a->dtype != b->dtype) return err_arg("operand dtypes differ");
  SX_CUDA(cudaSetDevice(ctx->device));
  sx_op op = new_op(ctx, kind, a->dtype, nrows, ncols);
  op->left = a;
  op->right = b;
  int rc = dev_alloc(&op->work, std::max<int64_t>(work_len, 1) * elt_size(a->dtype));
  if (rc) { delete op; return rc; }
  *out = op;
  return clear_error();
}

int sx_op_sum(sx_ctx ctx, sx_op a, sx_op b, sx_op* out) {
  if (!ctx || !a || !b || !out) return err_arg("null argument");
  if (a->nrows != b->nrows || a->ncols != b->ncols) {
    // interface.rs:308-313: ShapeMismatch{expected: a.shape(), found: b.shape()}
    return set_error(SX_ERR_SHAPE_MISMATCH,
                     "Shape mismatch: expected (" + std::to_string(a->nrows) + ", " + std::to_string(a->ncols) +
                         "), found (" + std::to_string(b->nrows) + ", " + std::to_string(b->ncols) + ")",
                     (uint64_t)a->nrows, (uint64_t)a->ncols, (uint64_t)b->nrows, (uint64_t)b->ncols);
  }
  return make_pair_op(ctx, SX_OP_SUM, a, b, a->nrows, a->ncols, a->nrows, out);
}

int sx_op_product(sx_ctx ctx, sx_op a, sx_op b, sx_op* out) {
  if (!ctx || !a || !b || !out) return err_arg("null argument");
  // interface.rs:360-366: DimensionMismatch{expected: a_cols, found: b_rows}
  if (a->ncols != b->nrows) return err_dim((uint64_t)a->ncols, (uint64_t)b->nrows);
  return make_pair_op(ctx, SX_OP_PRODUCT, a, b, a->nrows, b->ncols, b->nrows, out);
}

}  // extern "C"

namespace sx {
// y = y + t (interface.rs:340-344: a + b elementwise)
template <typename T>
__global__ void k_add_inplace(T* y, const T* __restrict__ t, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = add_rn(y[i], t[i]);
}
}  // namespace sx

extern "C" {

static bool has_adjoint(sx_op op) {
  switch (op->kind) {
    case SX_OP_HOST: return false;  // interface.rs:49-51 (the trait's default)
    case SX_OP_ILU0:                // preconditioners.rs:378-380
    case SX_OP_SSOR: return false;  // preconditioners.rs:189-191
    case SX_OP_SUM:
    case SX_OP_PRODUCT: return has_adjoint(op->left) && has_adjoint(op->right);  // :349, :399
    default: return true;
  }
}

int sx_op_has_adjoint(sx_op op, int* out) {
  if (!op || !out) return err_arg("null argument");
  *out = has_adjoint(op) ? 1 : 0;
  return SX_OK;
}

int sx_op_kind_of(sx_op op, int* kind) {
  if (!op || !kind) return err_arg("null argument");
  *kind = op->kind;
  return SX_OK;
}
int sx_op_shape(sx_op op, uint64_t* nrows, uint64_t* ncols) {
  if (!op) return err_arg("null op");
  if (nrows) *nrows = (uint64_t)op->nrows;
  if (ncols) *ncols = (uint64_t)op->ncols;
  return SX_OK;
}
int sx_op_dtype(sx_op op, int* dtype) {
  if (!op || !dtype) return err_arg("null argument");
  *dtype = op->dtype;
  return SX_OK;
}
int sx_op_destroy(sx_op op) {
  if (!op) return SX_OK;
  cudaSetDevice(op->device);
  cudaDeviceSynchronize();
  destroy_op_internal(op);
  return SX_OK;
}

// ----------------------------------------------------------------- matvec
int sx_op_matvec(sx_ctx ctx, sx_op op, const void* x, uint64_t x_len, void* y, sx_mem mem) {
  if (!ctx || !op) return err_arg("null argument");
  if (x_len != (uint64_t)op->ncols) return err_dim((uint64_t)op->ncols, x_len);
  SX_CUDA(cudaSetDevice(ctx->device));
  const size_t w = elt_size(op->dtype);
  if (mem == SX_MEM_DEVICE) {
    SX_CHECK(spmv_device(ctx, op, x, y, SX_SPMV_EXACT));
    SX_CUDA(cudaStreamSynchronize(ctx->stream));
    SX_CHECK(ic0_health(ctx, op));
    return clear_error();
  }
  void *dx = nullptr, *dy = nullptr;
  SX_CHECK(dev_alloc(&dx, std::max<int64_t>(op->ncols, 1) * w));
  int rc = dev_alloc(&dy, std::max<int64_t>(op->nrows, 1) * w);
  if (rc == SX_OK) {
    cudaMemcpyAsync(dx, x, op->ncols * w, cudaMemcpyHostToDevice, ctx->stream);
    rc = spmv_device(ctx, op, dx, dy, SX_SPMV_EXACT);
    if (rc == SX_OK) {
      cudaMemcpyAsync(y, dy, op->nrows * w, cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "matvec", __FILE__, __LINE__);
      else rc = ic0_health(ctx, op);
    }
  }
  dev_free(dx);
  dev_free(dy);
  return rc == SX_OK ? clear_error() : rc;
}

int sx_op_rmatvec(sx_ctx ctx, sx_op op, const void* x, uint64_t x_len, void* y, sx_mem mem) {
  if (!ctx || !op) return err_arg("null argument");
  switch (op->kind) {
    case SX_OP_CSR: {
      // interface.rs:281-285 transposes on every call; the device keeps the
      // transpose after the first call (identical arrays, identical result)
      if (x_len != (uint64_t)op->nrows) return err_dim((uint64_t)op->nrows, x_len);
      SX_CUDA(cudaSetDevice(ctx->device));
      SX_CHECK(ensure_transpose(ctx, op));
      return sx_op_matvec(ctx, op->transpose, x, x_len, y, mem);
    }
    case SX_OP_IDENTITY:
    case SX_OP_SCALED_IDENTITY:
    case SX_OP_DIAGONAL:
    case SX_OP_JACOBI:
    case SX_OP_IC0:
    case SX_OP_FSAI:
    case SX_OP_SYM_CSR:
      // self-adjoint operators: rmatvec = matvec (interface.rs:86-88,
      // :121-124, :164-167; preconditioners.rs:88-91; ic.rs:227-230)
      return sx_op_matvec(ctx, op, x, x_len, y, mem);
    case SX_OP_ZERO: {
      // interface.rs:211-218: zeros of length cols
      if (x_len != (uint64_t)op->nrows) return err_dim((uint64_t)op->nrows, x_len);
      SX_CUDA(cudaSetDevice(ctx->device));
      const size_t bytes = (size_t)op->ncols * elt_size(op->dtype);
      if (mem == SX_MEM_DEVICE) {
        SX_CUDA(cudaMemsetAsync(y, 0, bytes, ctx->stream));
        SX_CUDA(cudaStreamSynchronize(ctx->stream));
      } else {
        std::memset(y, 0, bytes);
      }
      return clear_error();
    }
    case SX_OP_SUM:
    case SX_OP_PRODUCT: {
      // interface.rs:332-345 and :382-395: both adjoints or OperationNotSupported;
      // (A + B)^H x = A^H x + B^H x, (A B)^H x = B^H (A^H x)
      if (!has_adjoint(op->left) || !has_adjoint(op->right))
        return set_error(SX_ERR_OPERATION_NOT_SUPPORTED,
                         "Operation not supported: adjoint not supported for one or both operators");
      if (x_len != (uint64_t)op->nrows) return err_dim((uint64_t)op->nrows, x_len);
      SX_CUDA(cudaSetDevice(ctx->device));
      const size_t w = elt_size(op->dtype);
      void *dx = nullptr, *t = nullptr, *dy = nullptr;
      int rc = SX_OK;
      do {
        if ((rc = dev_alloc(&dx, std::max<int64_t>(op->nrows, 1) * w))) break;
        if ((rc = dev_alloc(&dy, std::max<int64_t>(op->ncols, 1) * w))) break;
        const int64_t tlen = op->kind == SX_OP_SUM ? op->ncols : op->left->ncols;
        if ((rc = dev_alloc(&t, std::max<int64_t>(tlen, 1) * w))) break;
        SX_CUDA(cudaMemcpyAsync(dx, x, op->nrows * w,
                                mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                ctx->stream));
        if (op->kind == SX_OP_SUM) {
          if ((rc = sx_op_rmatvec(ctx, op->left, dx, op->nrows, dy, SX_MEM_DEVICE))) break;
          if ((rc = sx_op_rmatvec(ctx, op->right, dx, op->nrows, t, SX_MEM_DEVICE))) break;
          const int g = vec_grid(ctx, op->ncols);
          if (op->dtype == SX_F64)
            k_add_inplace<double><<<g, kBlock, 0, ctx->stream>>>((double*)dy, (const double*)t, op->ncols);
          else
            k_add_inplace<float><<<g, kBlock, 0, ctx->stream>>>((float*)dy, (const float*)t, op->ncols);
          ctx->launches++;
        } else {
          if ((rc = sx_op_rmatvec(ctx, op->left, dx, op->nrows, t, SX_MEM_DEVICE))) break;
          if ((rc = sx_op_rmatvec(ctx, op->right, t, op->left->ncols, dy, SX_MEM_DEVICE))) break;
        }
        SX_CUDA(cudaMemcpyAsync(y, dy, op->ncols * w,
                                mem == SX_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                ctx->stream));
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "composite rmatvec", __FILE__, __LINE__);
      } while (0);
      dev_free(dx);
      dev_free(t);
      dev_free(dy);
      return rc == SX_OK ? clear_error() : rc;
    }
    default:
      return set_error(SX_ERR_OPERATION_NOT_SUPPORTED,
                       "Operation not supported: adjoint not implemented for this operator");
  }
}

int sx_spmv_ex(sx_ctx ctx, sx_op a, const void* x_dev, void* y_dev, unsigned flags) {
  if (!ctx || !a || !x_dev || !y_dev) return err_arg("null argument");
  SX_CUDA(cudaSetDevice(ctx->device));
  return spmv_device(ctx, a, x_dev, y_dev, flags);
}

}  // extern "C"
