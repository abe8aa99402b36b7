// Device buffers and launch wrappers of the discrete adjoint.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "hg_state.hpp"

namespace hg {

// Adjoint accumulators and tables, device order.
struct AdjDev {
  double* gN = nullptr;        // [n] dL/dn per cell, accumulated over all stages
  double* gS0x = nullptr;      // [n] dL/dS0x per cell (S0 is linear in zb; mapped to zb at the end)
  double* gS0y = nullptr;
  double* gZb = nullptr;       // [n] dL/dzb through the exit-H ghost depth
  double* bfGradQ = nullptr;   // [nbf] per boundary face: sum_k w_k dF_k/dQ_inlet of the current stage
  double* bfGradTA = nullptr;  // [nbf] the same for the inlet conveyance total_A
  double* gQ = nullptr;        // [nInlet] dL/dQ_inlet, accumulated
  const int32_t* inletBf = nullptr;    // inlet CSR entry -> boundary face index
  const int32_t* inletUOff = nullptr;  // [nInlet+1] unique inlet cells per group
  const int32_t* inletUCell = nullptr;
  const double* inletUCoef = nullptr;  // sum over the cell's faces in the group of L^(5/3)
  double* loss = nullptr;              // [1] sum over steps and probes of (h - obs)^2
  // FP32-compensated path: per-cell sums of gN, gS0x, gS0y, gZb ([4][n]) as
  // unevaluated float pairs {hi, lo}, folded into the FP64 arrays at the end.
  float2* accF = nullptr;
  // FP32C boundary VJP (k_vjp_bnd_f32 beside the interior VJP, then
  // k_vjp_combine_f32): cells with at least one boundary face (device order),
  // their boundary-face terms of the current VJP {g_xi, g_hu, g_hv, g_n, g_zb},
  // the inlet (group, sum L^(5/3)) pairs of each (CSR), and the per-group sums
  // of the total_A cotangent.
  const int32_t* bndCells = nullptr;
  int32_t nBndCells = 0;
  float* bndG = nullptr;
  const int32_t* bndInOff = nullptr;
  const int32_t* bndInGrp = nullptr;
  const double* bndInCoef = nullptr;
  double* grpTA = nullptr;
  // {interior VJP tiles handed out past the first wave, interior CTAs
  // finished, boundary-VJP blocks finished}; zero between launches (the last
  // CTA or block out resets its counters).
  unsigned int* tileTicket = nullptr;
  // [nBndCells] the probe cell (ProbeCsr index) each boundary cell is, or -1.
  int32_t* bndProbe = nullptr;
  // Boundary faces folded into the pipelined interior VJP (no boundary or
  // combine launch per stage): every boundary face's flux Jacobian at each
  // stage state of a segment comes from one launch per segment
  // (k_bnd_jac_f32); the VJP of a stage contracts it with the cell's
  // cotangent.  6 float4 per face: float 7 r + d is dF_r / dp_d, r over
  // (F_xi, F_hu, F_hv), d over (own xi, hu, hv, n, zb, inlet Q, total_A).
  // bndJ: the current VJP's state.  The inlet groups' total_A and Q
  // cotangents are summed by the CTAs whose tiles hold inlet cells (tileGrp:
  // per tile a bit per group); the CTA of tile grpTile[g] adds group g's Q
  // cotangent to gQ.
  const float4* bndJ = nullptr;
  const int2* bfSlot = nullptr;       // [nbf] {device cell, slot}
  const float4* inletW = nullptr;     // [inlet CSR entries] {face as bits, cell as bits, len / area, 0}
  const uint32_t* tileGrp = nullptr;  // [interior VJP tiles]
  const int32_t* grpTile = nullptr;   // [nInlet]
  // Probe terms with the boundary faces folded: a segment's seeds (per step
  // with probes, per distinct probe cell) and loss sums come from one launch
  // (k_probe_seg_f32); the stage-1 VJP adds its step's seeds (probeSeed, null
  // for none) to the probe cells of each tile it computes (tileProbeOff/U: per
  // tile a CSR of distinct-probe-cell indices; probeCell: their cells).
  const float* probeSeed = nullptr;
  const int32_t* tileProbeOff = nullptr;
  const int32_t* tileProbeU = nullptr;
  const int32_t* probeCell = nullptr;
  // The gradients the caller asked for: the FP32C VJP accumulates the n or
  // the bed (S0, exit-H) terms only when wanted.
  int32_t wantN = 1, wantZb = 1;
  // A state-dependent Manning n (hg_set_manning_function: power law, sigmoid,
  // inverse, h_Umag_ks): n is then not a parameter but a function of each RHS
  // evaluation's input state, so each stage's dL/dn of a cell is taken back
  // into the cell's state cotangent through dn/d(h, qx, qy), and into the
  // function's parameters {n_lower, n_upper, k, h_mid} (per-cell FP64 sums
  // gResP [4][n]; the FP32C VJP adds into compensated pairs accRes, folded in
  // at the end).
  int32_t resChain = 0;
  // The FP32 VJP kernels as the VJP of the RHS alone (the stages of a Tsit5
  // step, which no clamp of the stage state follows): no dry-cell masks in
  // the VJP, its boundary terms or the probe seeds.
  int32_t noMask = 0;
  double* gResP = nullptr;
  float2* accRes = nullptr;
  // A UDE closure (hg_set_ude): udeChain = 1 when the network gives n
  // (ManningN_h, ManningN_h_Umag_ks; every dL/dn of a cell goes to the
  // network), 2 when it gives the friction magnitude F of the flow-resistance
  // closure (the friction term's dL/dF goes to the network; the inlet
  // conveyance's dL/dn stays a gradient of the cells' n).  The VJP kernels
  // store each stage's per-cell cotangent beta dL/d(n or F) in udeGn; the
  // network's VJP (launch_ude_vjp_*) then takes it back into the cells' state
  // cotangents and into gTheta [udeP], the parameters in hg_set_ude's order.
  int32_t udeChain = 0;
  int32_t udeP = 0;
  double* udeGn = nullptr;      // [n]
  double* gTheta = nullptr;     // [udeP], accumulated over the stages
  double* udePart = nullptr;    // [kUdeGrid * udeP] per-block partial sums
  double* udeS = nullptr;       // [2 kResMaxLayers] LayerNorm backward sums of the stage
  unsigned int* udeTicket = nullptr;
};

// Inlet groups the folded boundary VJP handles (tileGrp's bits).
constexpr int kFoldMaxGroups = 8;

// Grid of the network VJP (one warp per block, a fixed grid so that the
// per-block partial sums and their reduction have a fixed order).
constexpr int kUdeGrid = 1216;

// out_j = M(Q_j) (cSelf mu_j + cExtra extra_j + beta (J(Q)^T mu)_j), parameter
// gradients += beta (dR/dtheta)^T mu; M(Q_j) = 1 when cell j of Q is wet (the
// stage clamp), or always without mask (a state no clamp produced).
void launch_vjp_f64(const DevMesh& m, const AdjDev& a, const double* Q, const double* mu, const double* extra,
                    double* out, double cSelf, double cExtra, double beta, cudaStream_t st, bool mask = true);
// The UDE network's VJP of one stage (after that stage's VJP kernels):
// out += M(Q) (dn/dQ)^T udeGn, gTheta += (dn/dtheta)^T udeGn, the LayerNorm
// statistics taken over all cells when the network normalises over the batch.
// Needs the network's forward statistics of Q (launch_resistance_* of Q just
// before).  Returns the launches.
int launch_ude_vjp_f64(const DevMesh& m, const AdjDev& a, const double* Q, double* out, cudaStream_t st);
int launch_ude_vjp_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, float* out, cudaStream_t st);
// Inlet-Q conveyance terms of the same VJP (total_A couples all cells of a group).
void launch_inlet_adjoint_f64(const DevMesh& m, const AdjDev& a, const double* Q, double* out, double beta,
                              cudaStream_t st);
// Loss terms: forward (accumulate), adjoint (mu_xi[p] += M scale 2 (h - obs)).
void launch_probe_loss_f64(const DevMesh& m, const AdjDev& a, const double* Q, const int32_t* probes,
                           const double* obs, int32_t nprobe, cudaStream_t st);
void launch_probe_adjoint_f64(const DevMesh& m, const double* Q, double* mu, const int32_t* probes,
                              const double* obs, int32_t nprobe, double scale, cudaStream_t st, bool mask = true);
// FP32-compensated path: the same with packed FP32 states and FP32 cotangents.
// The whole VJP of one stage, inlet-Q terms included, on st: the
// boundary-face kernel, the interior kernel beside it (a programmatic
// dependent launch), then the combine kernel.  beta = betaD as FP32.
// Returns the launches made.
// The folded boundary VJP (see AdjDev::bndJ): usable with the pipelined
// interior kernel, at most kFoldMaxGroups inlet groups and the tables built.
bool vjp_fold_usable(const DevMesh& m, const AdjDev& a, StateF32 Q);
// The boundary faces' flux Jacobians of nStates consecutive FP32C states
// (state s: records X + s n, inlet totals tot + s totStride) into J.
int launch_bnd_jac_f32(const DevMesh& m, const AdjDev& a, const float4* X, int nStates, const double* tot,
                       size_t totStride, float4* J, cudaStream_t st);
// The probe seeds (seeds + (s - sFirst) nCells, per distinct probe cell) and
// loss sums (lossPart[s - 1]) of steps s = sFirst .. sFirst + nSteps - 1 of a
// segment starting at step s0: the state after step s - 1 has records
// X + (s - s0) n, its observations obs + (s - 1) np.
int launch_probe_seg_f32(const DevMesh& m, const float4* X, int s0, int sFirst, int nSteps,
                         const struct ProbeCsr& pc, const int32_t* probes, const double* obs, int32_t np,
                         double scale, float* seeds, double* lossPart, cudaStream_t st);
// loss += lossPart[s - 1] for s = sLast down to 1 (the reverse sweep's order).
int launch_loss_parts(const AdjDev& a, const double* lossPart, int sLast, cudaStream_t st);
// One stage's VJP with the boundary faces folded in (a.bndJ of Q): the
// interior kernel, and the probe kernel when pj has probes.
int launch_vjp_f32_folded(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra,
                          float* out, float cSelf, float cExtra, double beta, cudaStream_t st,
                          const struct ProbeJob* pj);
int launch_vjp_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra, float* out,
                   float cSelf, float cExtra, double betaD, cudaStream_t st, const struct ProbeJob* pj = nullptr);
// Probes grouped by cell: cell[u] (distinct, device order) holds probes idx[off[u] .. off[u+1]).
struct ProbeCsr {
  const int32_t* cell = nullptr;
  const int32_t* off = nullptr;
  const int32_t* idx = nullptr;
  const int32_t* isBnd = nullptr;   // [nCells] 1: a boundary cell (its seed comes with the combine)
  int32_t nCells = 0;
};
// The probe terms of the VJP's state, done by the stage-1 VJP's combine launch
// (np = 0: none).
struct ProbeJob {
  ProbeCsr pc;
  const int32_t* probes = nullptr;
  const double* obs = nullptr;
  int32_t np = 0;
  double scale = 0.0;
};
// The probe loss of state Q (into a.loss) and its seed into mu (one kernel).
void launch_probe_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, float* mu, const ProbeCsr& pc,
                      const int32_t* probes, const double* obs, int32_t nprobe, double scale, cudaStream_t st);
// Final-state inversion loss (swe_2D_inversion.jl:383-431), device order:
//   WSE term  sum_c ((h_c + zbw_c - wse_c) / wseDen)^2 / n,  h = xi + hstill
//   uv term   sum_c ((qx_c / (h_c + eps) - u_c)^2 + (qy_c / (h_c + eps) - v_c)^2) / velScale^2 / n
// with eps = sqrt(eps(Float64)).  launch_final_loss_* add the loss's gradient
// w.r.t. the final state to mu (masked by the last stage's clamp, like the
// probe terms), write dL/dWSE per cell to dWse (the direct term of an active
// zb parameter) and the two sums to parts[0..1] (deterministic reduction).
constexpr int kFinalLossBlocks = 1024;
struct FinalLossDev {
  const double* wse = nullptr;   // [n] or null: no WSE term
  const double* u = nullptr;     // [n] u, v or null: no velocity term
  const double* v = nullptr;
  const double* zbw = nullptr;   // [n] zb of WSE_pred
  const double* lam = nullptr;   // [3n] or null: a cotangent of the final state added to the seed
  double wseDen = 1.0;           // WSE_truth range + eps
  double velScale = 1.0;
  double invN = 1.0;
  double* dWse = nullptr;        // [n]
  int32_t mask = 1;              // 1: cells at h_small (clamped by the last stage) take no seed
  double* parts = nullptr;       // [2]
  double* partials = nullptr;    // [2 * kFinalLossBlocks]
  unsigned int* ticket = nullptr;
};
void launch_final_loss_f64(const DevMesh& m, const FinalLossDev& f, const double* Q, double* mu, cudaStream_t st);
void launch_final_loss_f32(const DevMesh& m, const FinalLossDev& f, StateF32 Q, float* mu, cudaStream_t st);
// gN, gS0x, gS0y, gZb += the FP32 pair accumulators (accF).
void launch_fold_accumulators_f32(const DevMesh& m, const AdjDev& a, cudaStream_t st);
// dL/dzb = S0 transpose (Green-Gauss of face averages) applied to dL/dS0, plus the direct term.
void launch_zb_gradient(const DevMesh& m, const AdjDev& a, double* gzb, cudaStream_t st);
// out4[k] = sum over cells of gResP[k] (a state-dependent n's parameter gradient).
void launch_res_param_sum(const AdjDev& a, int n, double* out4, cudaStream_t st);

}  // namespace hg
