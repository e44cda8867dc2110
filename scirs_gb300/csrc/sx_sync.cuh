// Flag-based dependency waits shared by the triangular factorisations and
// solves (IC(0), ILU(0), SSOR): rows are handed to warps in dependency-level
// order through an atomic counter, a row waits only on rows handed out
// before it, and every wait is bounded.  A wait that gives up raises the
// abort flag, which ends every other wait at once.
#pragma once

#include "sx_internal.h"

namespace sx {
namespace {


__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_flag(const int* p) { return *(volatile const int*)p; }
// acquire load: later loads see what the publisher wrote before its release
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until *flag != 0; false if the wait was abandoned (abort raised or
// the context's limit of `limit_ns` per wait passed; 2 s by default).  Spins
// without sleeping first: the wait sits on the critical path of the
// triangular solves, one wait per dependency level.
__device__ bool wait_flag(const int* flag, int* abort, unsigned long long limit_ns) {
  if (ld_acquire(flag)) return true;
  const unsigned long long t0 = globaltimer();
  for (unsigned it = 1;; ++it) {
    if (ld_acquire(flag)) return true;
    if ((it & 63u) == 0) {
      if (ld_flag(abort)) return false;
      if (globaltimer() - t0 > limit_ns) {
        atomicExch(abort, 1);
        return false;
      }
    }
    if (it > 4096u) __nanosleep(128);
  }
}

// release store: the row's result is visible before its flag
__device__ __forceinline__ void publish(int* flag) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(flag), "r"(1) : "memory");
}

template <typename T>
__device__ __forceinline__ T ldv(const T* p) { return __ldcg(p); }

// ---- building L: lower entries (col <= row) in storage order (ic.rs:32-49)
__global__ void k_lower_count(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              int64_t n, int32_t* cnt) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t c = 0;
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) c += idx[k] <= (int32_t)r;
    cnt[r] = c;
  }
}

template <typename T>
__global__ void k_lower_copy(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const T* __restrict__ val, int64_t n, const int32_t* __restrict__ lp,
                             int32_t* li, T* lv) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t o = lp[r];
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k)
      if (idx[k] <= (int32_t)r) { li[o] = idx[k]; lv[o] = val[k]; ++o; }
  }
}

}  // namespace
}  // namespace sx
