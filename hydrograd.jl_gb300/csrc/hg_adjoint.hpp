// Discrete adjoint of the SSP-RK2 time stepping (host driver in hg_adjoint.cpp,
// kernels in hg_adjoint.cu).
#pragma once
#include <cstdint>

struct hg_ctx;

namespace hg {

int adjoint_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                          const int32_t* probe_cells, const double* obs, int32_t n_probe, double* loss,
                          double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final);
void adjoint_release(hg_ctx* ctx);

}  // namespace hg
