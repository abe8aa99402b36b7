// The context behind the opaque hg_ctx handle.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hg_mesh.hpp"
#include "hg_state.hpp"
#include "hydrograd_gb.h"

namespace hg {
constexpr int kGraphSteps = 50;   // steps per captured CUDA graph
struct AdjointBuffers;
}  // namespace hg

struct hg_ctx {
  hg::HostMesh hm;
  hg_consts k{};
  int32_t precision = HG_FP64;
  int32_t device = 0;
  int32_t n = 0;
  std::vector<int> perm, inv;   // perm[device id] = caller id
  // Ensemble members (hg_ensemble_create): cell, inlet-Q and exit-H boundary
  // offsets per member in the caller's order ([n_members + 1]; empty otherwise).
  std::vector<int32_t> memberCellOff, memberInletOff, memberExitOff;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  hg::DevMesh dm;
  hg::DevScalars ds;
  // Parameters (caller order, FP64 host copies)
  std::vector<double> zbCell, hstill, manning, s0x, s0y, inletQ, exitWse;
  // FP32 packed cell records (device order), host copies kept alive across async uploads
  std::vector<float4> h_CP, h_CS;
  std::vector<float> h_area;   // device order
  // Exit-H boundary faces: boundary-face index, caller cell id, group; and the
  // FP32 path's (WSE - zb) - hstill per boundary face, formed in FP64.
  std::vector<int32_t> exitBf, exitCell, exitGrp;
  std::vector<float> h_bfExitRel;
  float* d_bfExitRel = nullptr;
  // Writable device parameter arrays
  double *d_hst = nullptr, *d_zb = nullptr, *d_man = nullptr, *d_s0x = nullptr, *d_s0y = nullptr;
  float4 *d_CP = nullptr, *d_CS = nullptr;
  double *d_inletQ = nullptr, *d_exitWse = nullptr, *d_totalA = nullptr;
  int32_t* d_perm = nullptr;
  const int32_t* slotNb = nullptr;
  // State
  double *QA = nullptr, *QB = nullptr, *Quser = nullptr;
  float4 *XA = nullptr, *XB = nullptr;   // FP32 path state records
  float2 *XQA = nullptr, *XQB = nullptr;
  void* flushBuf = nullptr;
  size_t flushBytes = 0;
  bool cflPrimed = false;
  // Fused FP32 stepping: conveyance totals of the resident state (tot) and of
  // the stage buffer (tot + kMaxFusedInlets), per-block partials, last-block ticket.
  double* d_tot = nullptr;
  double* d_partials = nullptr;
  unsigned int* d_ticket = nullptr;
  int32_t* d_blockSlot = nullptr;   // slot of each stage block that holds inlet cells, else -1
  int32_t nSlots = 0;
  int32_t nWarps = 0;   // warps of the tiles holding inlet cells (StageFuse::nWarps)
  int parity = 0;                   // CFL-minimum buffer the next fused step reads
  int graphParity = 0;              // parity the captured graph starts (and ends) with
  // Captured graph of kGraphSteps steps
  cudaGraphExec_t graphExec = nullptr;
  bool graphValid = false, graphCflMode = false;
  double graphCfl = 0.0;
  int64_t graphLaunches = 0;
  bool stageTuned = false;          // hg_autotune has chosen dm.stageKernel / dm.stageVariant
  int32_t stageFamily = 0;          // candidates of the autotuner: 0 gather, pipe, tma; 1 face (see autotune_stage)
  int32_t tuneSource = 0;           // where the choice came from: 0 default, 1 timed, 2 cache, 3 forced
  uint64_t meshSig = 0;             // hash of the device-order face tables (autotune cache key)
  // The last gradient call's gradient w.r.t. the parameters {n_lower, n_upper,
  // k, h_mid} of a state-dependent n (hg_resistance_grad).
  double resGrad[4] = {0.0, 0.0, 0.0, 0.0};
  // UDE closure: its parameter count and the last gradient's dL/dtheta
  int32_t udeParams = 0;
  std::vector<double> udeGrad;
  int64_t launches = 0;
  hg::AdjointBuffers* adj = nullptr;
  // Adjoint stage-state tape (hg_set_adjoint_tape): -1 automatic budget, 0 the
  // caller's checkpoint spacing exactly, > 0 a budget in bytes.
  int64_t adjTapeBytes = -1;
  int32_t adjIntegrator = 0;        // the steps the adjoint differentiates: 0 SSP-RK2, 1 fixed-step Tsit5
  std::vector<double> adjSteps;     // hg_set_adjoint_steps: the Tsit5 adjoint's step sizes (empty: dt each)
  std::vector<double> tsit5Steps;   // the step sizes the last hg_integrate_tsit5 accepted (hg_tsit5_steps)
  // State-dependent resistance (hg_set_manning_function / hg_set_ude): device
  // buffers, allocated on first use; dm.res points into them.
  double *d_resKs = nullptr, *d_resW = nullptr, *d_resStats = nullptr, *d_resPartials = nullptr, *d_fres = nullptr;
  void* d_resAct = nullptr;   // the network's cached hidden-layer values (ResDev::hid / hidF)
  size_t resActBytes = 0;
  float *d_resWf = nullptr, *d_fresF = nullptr;
  unsigned int* d_resTicket = nullptr;
  // Inlet-Q hydrographs (hg_set_inlet_hydrograph): per group its times then
  // its discharges; device copies (dm.hydro*), capacity in points.
  std::vector<std::vector<double>> hydro;
  int32_t* d_hydroOff = nullptr;
  double *d_hydroT = nullptr, *d_hydroQ = nullptr;
  size_t hydroCap = 0;
  std::string err;
  ~hg_ctx();
};

int ctx_setup_device(hg_ctx* c);
