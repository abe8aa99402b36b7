// Discrete adjoint of the SSP-RK2 time stepping (host driver in hg_adjoint.cpp,
// kernels in hg_adjoint.cu).
#pragma once
#include <cstdint>

struct hg_ctx;

namespace hg {

// Observations of the final-state inversion loss (swe_2D_inversion.jl:383-431),
// caller order: WSE_truth (or null), u_truth and v_truth (or null), and the zb
// of WSE_pred = h + zb (null: the context's zb, an active zb parameter whose
// direct term then enters g_zb).
struct FinalObs {
  const double* wse = nullptr;
  const double* u = nullptr;
  const double* v = nullptr;
  const double* zbw = nullptr;
  const double* lam = nullptr;   // [3n] cotangent of the final state (caller's cell order), added to the seed
};

// loss = the probe misfit (mean over steps and probes) + the final-state loss
// of fo (if given); parts (if given) = {final loss, its WSE term, its uv term}.
int adjoint_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                          const int32_t* probe_cells, const double* obs, int32_t n_probe, double* loss,
                          double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final,
                          const FinalObs* fo = nullptr, double* parts = nullptr);
// Mean duration of n launches of the FP32C interior VJP kernel (boundary
// faces folded, the stage-2 form: out = 0.5 mu + beta J^T mu) on the resident
// state, CUDA events on the context's stream, L2 flushed between launches
// when flushL2.
int adjoint_time_vjp(hg_ctx* ctx, int32_t n, int32_t flushL2, double* avgMs);
void adjoint_release(hg_ctx* ctx);
// Free the stage-state tape and checkpoint buffers (the next gradient call allocates what it needs).
void adjoint_release_tape(hg_ctx* ctx);

}  // namespace hg
