// Autotuner of launch shapes.  A kernel family exposes a small set of
// candidate shapes (threads per block, blocks per SM, ...); the first call
// for a given problem key times every candidate on a bounded sample of the
// real work with CUDA events on the context's stream and keeps the fastest
// in the context (sx_ctx_s::tuned), so later calls with the same key launch
// it directly.  The key folds the family and bucketed size statistics, the
// way a tuning cache keyed by kernel and problem size does
// (scirs2-core/src/gpu/auto_tuning.rs:265-390).  SX_TUNE=0 turns tuning off
// (the family's first candidate is used); SX_TUNE_FORCE=<index> forces one.
#pragma once

#include <cstdlib>
#include <cstring>
#include <functional>

#include "sx_internal.h"

namespace sx {

enum TuneFamily : uint32_t { TUNE_BATCHED_PCG = 1 };

// log2 bucket of a count (0 below 2)
inline uint32_t tune_bucket(double v) {
  uint32_t b = 0;
  while (v >= 2.0 && b < 63) { v *= 0.5; ++b; }
  return b;
}

inline uint64_t tune_key(TuneFamily f, uint32_t a, uint32_t b, uint32_t c) {
  return ((uint64_t)f << 48) | ((uint64_t)(a & 0xFFFF) << 32) | ((uint64_t)(b & 0xFFFF) << 16) | (c & 0xFFFF);
}

// Picks one of ncand candidates.  run(i) enqueues candidate i's sample on
// the context stream; the sample must be safe to repeat (the real work
// redoes it afterwards).
inline int tune_pick(sx_ctx ctx, uint64_t key, int ncand, const std::function<int(int)>& run, int* chosen) {
  *chosen = 0;
  if (const char* f = std::getenv("SX_TUNE_FORCE")) {
    const int k = std::atoi(f);
    if (k >= 0 && k < ncand) *chosen = k;
    return SX_OK;
  }
  if (const char* t = std::getenv("SX_TUNE"))
    if (std::strcmp(t, "0") == 0) return SX_OK;
  auto it = ctx->tuned.find(key);
  if (it != ctx->tuned.end() && (int)it->second < ncand) {
    *chosen = (int)it->second;
    return SX_OK;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SX_CUDA(cudaEventCreate(&e0));
  SX_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int rc = SX_OK;
  for (int i = 0; i < ncand && rc == SX_OK; ++i) {
    // one untimed run (first-launch costs), then the timed one
    if ((rc = run(i)) != SX_OK) break;
    cudaEventRecord(e0, ctx->stream);
    if ((rc = run(i)) != SX_OK) break;
    cudaEventRecord(e1, ctx->stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "autotune", __FILE__, __LINE__);
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      *chosen = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == SX_OK) ctx->tuned[key] = (uint32_t)*chosen;
  return rc;
}

}  // namespace sx
