// Roofline probe: the random-gather rate of this GPU.
//
// SpMV on a matrix with scattered columns (a power-law graph) reads x[col]
// once per nonzero at an unpredictable address: 32 separate sector requests
// per warp instruction.  Their rate, not HBM, bounds such matrices when x
// stays in L2.  The probe measures it the same way: int32 indices uniform in
// [0, n), streamed with coalesced loads, each gathering one element of an
// L2-resident vector of n elements, every load of a thread issued before the
// first is used.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "sx_internal.h"
#include "sx_kernels.cuh"

namespace sx {

// uniform indices in [0, n) from a counter hash (splitmix64 finaliser)
__global__ void k_probe_indices(int32_t* idx, int64_t m, int64_t n, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += stride) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    idx[k] = (int32_t)(z % (uint64_t)n);
  }
}

template <typename T, int U>
__global__ void __launch_bounds__(kBlock, 4) k_probe_gather(const int32_t* __restrict__ idx, const T* __restrict__ x,
                                                            int64_t m, T* out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  T acc = T(0);
  for (int64_t k0 = tid; k0 < m; k0 += stride * U) {
    int32_t c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = k0 + u * stride;
      c[u] = k < m ? __ldcs(idx + k) : 0;
    }
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = __ldg(x + c[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) acc += v[u];
  }
  out[tid] = acc;
}

template <typename T>
static int probe_gather(sx_ctx ctx, int64_t n, int64_t m, double* rate) {
  constexpr auto kern = k_probe_gather<T, 8>;
  int nb = 0;
  SX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlock, 0));
  const int64_t grid = (int64_t)ctx->num_sms * std::max(nb, 1);
  int32_t* idx = nullptr;
  T* x = nullptr;
  T* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SX_OK;
  do {
    if ((rc = dev_alloc((void**)&idx, m * 4))) break;
    if ((rc = dev_alloc((void**)&x, n * sizeof(T)))) break;
    if ((rc = dev_alloc((void**)&out, grid * kBlock * sizeof(T)))) break;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "probe events", __FILE__, __LINE__);
      break;
    }
    cudaMemsetAsync(x, 0, n * sizeof(T), ctx->stream);
    k_probe_indices<<<vec_grid(ctx, m), kBlock, 0, ctx->stream>>>(idx, m, n, 0x5EEDull);
    ctx->launches++;
    float best = 0.f;
    for (int r = 0; r < 4; ++r) {
      // a short pass first: x in L2, as it is after an SpMV's first rows
      kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(idx, x, std::min<int64_t>(m, grid * kBlock * 8), out);
      cudaEventRecord(e0, ctx->stream);
      kern<<<(unsigned)grid, kBlock, 0, ctx->stream>>>(idx, x, m, out);
      cudaEventRecord(e1, ctx->stream);
      ctx->launches += 2;
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "gather probe", __FILE__, __LINE__);
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r == 0 || ms < best) best = ms;
    }
    if (rc == SX_OK) *rate = (double)m / (best * 1e-3);
  } while (0);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dev_free(idx);
  dev_free(x);
  dev_free(out);
  return rc;
}

}  // namespace sx

using namespace sx;

extern "C" int sx_probe_gather_rate(sx_ctx ctx, sx_dtype dtype, uint64_t n, uint64_t m, double* gathers_per_s) {
  if (!ctx || !gathers_per_s) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (n == 0 || m == 0 || n > (uint64_t)INT32_MAX || m > (1ull << 32))
    return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: probe sizes");
  if (dtype != SX_F32 && dtype != SX_F64) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: dtype");
  SX_CUDA(cudaSetDevice(ctx->device));
  const int rc = dtype == SX_F32 ? probe_gather<float>(ctx, (int64_t)n, (int64_t)m, gathers_per_s)
                                 : probe_gather<double>(ctx, (int64_t)n, (int64_t)m, gathers_per_s);
  return rc == SX_OK ? clear_error() : rc;
}
