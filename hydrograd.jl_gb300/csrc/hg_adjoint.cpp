// Host driver of the discrete adjoint (checkpointed SSP-RK2).
#include "hg_adjoint.hpp"

#include "hg_ctx.hpp"

namespace hg {

struct AdjointBuffers {};

int adjoint_loss_and_grad(hg_ctx* ctx, const double*, int32_t, double, int32_t, const int32_t*, const double*, int32_t,
                          double*, double*, double*, double*, double*) {
  ctx->err = "hg_loss_and_grad: not available in this build";
  return HG_ERR_UNSUPPORTED;
}

void adjoint_release(hg_ctx* ctx) {
  delete ctx->adj;
  ctx->adj = nullptr;
}

}  // namespace hg
