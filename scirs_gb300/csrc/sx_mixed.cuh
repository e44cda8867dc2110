// FP64 residual pieces shared by the two mixed-precision CG drivers.
#pragma once

#include "sx_launch.cuh"

namespace sx {

struct IrNorms {
  double rr, bb, rnorm, inv_rnorm;
};

// y = b - A x in FP64 with ||y||^2 and ||b||^2 fused
struct EpiIrResid {
  static constexpr bool kBanded = true;
  const double* b;
  IrNorms* norms;
  static constexpr bool kReduce = true;
  __device__ bool skip() const { return false; }
  __device__ double out(int64_t i, double ax) const { return sub_rn(b[i], ax); }
  __device__ void acc(int64_t i, double y, Acc3<double>& a) const {
    a.a += y * y;
    a.b += b[i] * b[i];
  }
  __device__ void finish(const Acc3<double>& t) const {
    norms->rr = t.a;
    norms->bb = t.b;
    // one square root and one division here instead of one per element
    norms->rnorm = sqrt(t.a);
    norms->inv_rnorm = 1.0 / norms->rnorm;
  }
};

// FP32 CG with FP64 residual replacement (sx_krylov.cu).  b, x, r are FP64
// device vectors (x holds x0 on entry and the solution on return); norms is
// one device IrNorms.
int cg_mixed_replace(sx_ctx ctx, sx_op a64, sx_op a32, sx_op m, const double* b, double* x, double* r,
                     IrNorms* norms, const sx_ir_options* opt, uint64_t* outer, uint64_t* inner,
                     double* rel, int* converged);

}  // namespace sx
