// FP64 true relative residual ||b - A x|| / ||b|| without any device
// allocation.
//
// Some callers cannot allocate device memory while they run: a host
// framework that owns every byte of GPU memory through its own pool (and
// forbids cudaMalloc outside it), a real-time or safety-critical loop where an
// allocation could stall or fail, or code running between the capture of
// other work whose memory plan is fixed.  They still need the FP64 residual
// check that ends a mixed-precision solve.  sx_true_rel_residual allocates a
// residual vector and reduction space per call; this variant computes the
// same residual entries (bit-identical: the same per-row order) and their
// norms with its reduction partials, ticket counter and totals in a
// file-scope device array, and takes b and x as device pointers.  Its
// reduction tree is one row per thread, so the norms agree with the
// allocating entry point's (whose tree follows the SpMV's work split) to the
// rounding of the summation order.
//
// Limits and sharing:
//  - at most kNoAllocMaxRows rows (the scratch holds one partial pair per
//    256-row block); larger matrices are rejected with SX_ERR_VALUE;
//  - every GPU that loads this library holds the array (3 * 65,536 + 6
//    doubles = 1,572,912 bytes, about 1.5 MiB) until exit;
//  - the array is shared by every call: calls that overlap on the GPU (two
//    streams, two host threads) race on it and must be serialised by the
//    caller.  Each call clears the ticket counter it relies on.
//  - the first call on a device looks up the array's device address there
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture.

#include <cmath>
#include <string>

#include "sx_internal.h"
#include "sx_kernels.cuh"

namespace {

constexpr int64_t kNoAllocMaxBlocks = 65536;
constexpr int64_t kNoAllocMaxRows = kNoAllocMaxBlocks * sx::kBlock;  // 16,777,216
// layout (doubles): [0, 3*kNoAllocMaxBlocks) block partials, then the
// ticket counter (as unsigned int) and the two totals
constexpr int64_t kCounterSlot = 3 * kNoAllocMaxBlocks;
constexpr int64_t kTotalsSlot = kCounterSlot + 2;
constexpr int64_t kScratchDoubles = kTotalsSlot + 4;

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// One thread per row: r_i = b_i - sum_k a_ik x_k (products and sums rounded
// in storage order, as the exact SpMV), then ||r||^2 and ||b||^2 through the
// same per-block / last-block reduction as the allocating entry point.
__global__ void __launch_bounds__(sx::kBlock) k_residual_norms_noalloc(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const double* __restrict__ vals, const double* __restrict__ b, const double* __restrict__ x,
    int64_t nrows, double* scratch) {
  const int64_t row = (int64_t)blockIdx.x * sx::kBlock + threadIdx.x;
  sx::Acc3<double> a{0.0, 0.0, 0.0};
  if (row < nrows) {
    double acc = 0.0;
    for (int32_t k = indptr[row]; k < indptr[row + 1]; ++k)
      acc = sx::add_rn(acc, sx::mul_rn(vals[k], __ldg(x + indices[k])));
    const double r = sx::sub_rn(b[row], acc);
    a.a += r * r;
    a.b += b[row] * b[row];
  }
  sx::Acc3<double> tot;
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kCounterSlot);
  if (sx::grid_reduce3(a, scratch, counter, tot) && threadIdx.x == 0) {
    scratch[kTotalsSlot + 0] = tot.a;
    scratch[kTotalsSlot + 1] = tot.b;
  }
}

int scratch_for_device(int device, double** out) {
  if (device < 0 || device >= kMaxDevices)
    return sx::set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: device id out of range");
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return sx::cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
    g_scratch_ptr[device] = (double*)p;
  }
  *out = g_scratch_ptr[device];
  return SX_OK;
}

}  // namespace

extern "C" int sx_true_rel_residual_noalloc(sx_ctx ctx, sx_op a64, const double* b_dev,
                                            const double* x_dev, double* out) {
  if (!ctx || !a64 || !out || !b_dev || !x_dev)
    return sx::set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a64->kind != SX_OP_CSR || a64->dtype != SX_F64)
    return sx::set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: needs an FP64 CSR matrix");
  const int64_t n = a64->nrows;
  if (n > kNoAllocMaxRows)
    return sx::set_error(SX_ERR_VALUE, "Value error: the allocation-free residual supports at most " +
                                           std::to_string(kNoAllocMaxRows) + " rows, got " +
                                           std::to_string(n));
  SX_CUDA(cudaSetDevice(ctx->device));
  double* scratch = nullptr;
  SX_CHECK(scratch_for_device(ctx->device, &scratch));
  // the ticket counter and the totals must start at zero
  SX_CUDA(cudaMemsetAsync(scratch + kCounterSlot, 0, 6 * sizeof(double), ctx->stream));
  const int64_t blocks = n > 0 ? (n + sx::kBlock - 1) / sx::kBlock : 1;
  k_residual_norms_noalloc<<<(unsigned)blocks, sx::kBlock, 0, ctx->stream>>>(
      a64->csr.indptr, a64->csr.indices, (const double*)a64->csr.vals, b_dev, x_dev, n, scratch);
  ctx->launches++;
  SX_CUDA(cudaGetLastError());
  double tot[2] = {0.0, 0.0};
  SX_CUDA(cudaMemcpyAsync(tot, scratch + kTotalsSlot, sizeof(tot), cudaMemcpyDeviceToHost, ctx->stream));
  SX_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = std::sqrt(tot[0]) / std::sqrt(tot[1]);
  return sx::clear_error();
}
