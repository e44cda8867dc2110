// IC(0) preconditioner (scirs2-sparse/src/linalg/ic.rs:15-230).
#include "sx_internal.h"

namespace sx {

struct IC0Dev {
  int dummy = 0;
};

void ic0_destroy(IC0Dev* p) { delete p; }

int ic0_apply(sx_ctx, sx_op, const void*, void*) {
  return set_error(SX_ERR_NOT_IMPLEMENTED, "Feature not implemented: IC0 apply");
}

}  // namespace sx

extern "C" int sx_precond_ic0(sx_ctx, sx_op, int, sx_op*) {
  return sx::set_error(SX_ERR_NOT_IMPLEMENTED, "Feature not implemented: IC0");
}
