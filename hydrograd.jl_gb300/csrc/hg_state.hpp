// Device-side data of a context and the launch wrappers shared by the host
// code (hg_capi.cpp) and the kernels (hg_forward.cu, hg_adjoint.cu).
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace hg {

// Mesh and parameters in device memory, cells in the device (renumbered) order.
// Slot-major face tables: entry [k * n + c] is edge slot k of cell c.
// State-dependent flow resistance (hg_resistance.cu).  Kinds: Manning's n as a
// function of the state (process_ManningN_2D.jl:102-213) and the UDE closures
// (process_ManningN_2D.jl:216-273: n from a network; process_FlowResistance_UDE.jl:3-45:
// the friction magnitude from a network).  Before every RHS evaluation the
// resistance kernels recompute, from that evaluation's input state, the
// per-cell n (DevMesh::man and CP.w, read by the friction and the inlet-Q
// conveyance) or the friction magnitude (fres / fresF).
enum ResKind : int32_t {
  kResConstant = 0, kResPowerLaw = 1, kResSigmoid = 2, kResInverse = 3, kResHUmagKs = 4,
  kResUdeManningH = 5, kResUdeManningHUmagKs = 6, kResUdeFlowResistance = 7
};
constexpr int kResMaxLayers = 4;     // hidden Dense + LayerNorm layers
constexpr int kResMaxWidth = 16;     // neurons per hidden layer
constexpr int kResMaxInputs = 3;
constexpr int kResBlock = 256;       // threads of a resistance block (one cell each)
// Blocks of a LayerNorm statistics pass over n cells, at most (four partials
// each: the block's sum, squared deviations about its mean, its count of
// values, that mean).
constexpr int64_t res_stat_blocks(int64_t n) { return (n + kResBlock - 1) / kResBlock; }
struct ResDev {
  int32_t kind = kResConstant;
  double p[4] = {0.0, 0.0, 0.0, 0.0};   // n_lower, n_upper, k, h_mid
  const double* ks = nullptr;           // [n] roughness height
  // network (Lux order: per hidden layer Dense weight (out x in, column-major),
  // bias, LayerNorm scale, bias; then the output Dense weight, bias)
  int32_t inDim = 0, nHidden = 0, overBatch = 1;
  int32_t width[kResMaxLayers] = {0, 0, 0, 0};
  int32_t act[kResMaxLayers] = {0, 0, 0, 0};
  const double* w = nullptr;
  const float* wf = nullptr;
  double outLo = 0.0, outHi = 1.0, lnEps = 1e-5;
  // input normalisation bounds: [0] h, [1] Umag (or the velocity magnitude of
  // the flow-resistance closure), [2] ks
  double lo[kResMaxInputs] = {0.0, 0.0, 0.0}, hi[kResMaxInputs] = {1.0, 1.0, 1.0};
  double* stats = nullptr;              // [2 * kResMaxLayers] LayerNorm mean, variance over all cells
  double* partials = nullptr;           // [4 res_stat_blocks(n)]
  unsigned int* ticket = nullptr;
  double* fres = nullptr;               // [n] friction magnitude (flow-resistance closure), FP64 path
  float* fresF = nullptr;               // the same, FP32 path
  // LayerNorm over the batch: the hidden layers' post-activation values of
  // every cell, [sum of widths][n] (layer l's rows from the sum of the widths
  // before it), kept by the statistics passes so that each pass starts from
  // the layer before instead of the inputs (FP64 path: hid; FP32 path: hidF)
  double* hid = nullptr;
  float* hidF = nullptr;
};

struct DevMesh {
  int32_t n = 0;        // cells
  int32_t nslot = 0;    // max faces per cell
  int32_t nbf = 0;      // boundary faces
  int32_t nInlet = 0, nExit = 0;
  int32_t riemann = 0;  // face Riemann solver: 0 Roe, 1 HLL (hg_set_riemann_solver)
  const int32_t* nb = nullptr;       // [nslot*n] neighbour (>=0), -1-bf (boundary face bf), INT32_MIN (none)
  const double* snx = nullptr;       // [nslot*n] outward unit normal x
  const double* sny = nullptr;
  const double* slen = nullptr;      // [nslot*n] edge length
  const float4* SL = nullptr;        // FP32 path: [nslot*n] {nx, ny, L, nb as bits} (see hg_f32.cuh)
  // Pipelined FP32 stage (meshes of degree <= 4): the slot records with the
  // neighbour as a tile-local index (own cells [0, kStageBlockF32), halo
  // cells kStageBlockF32 + j), and each tile's halo: the out-of-tile
  // neighbour cells, kHaloMax per tile, -1 padded.  Null when some tile has
  // a larger halo.
  const float4* SLp = nullptr;
  const int32_t* halo = nullptr;
  // Face-once FP32 stage (k_stage_face_f32; meshes of degree <= 4 whose
  // tiles' halos fit): per tile of kStageBlockF32 cells its faces, each listed
  // once (FL[FLoff[t] .. FLoff[t + 1]): {nx, ny, L of side a, packed ids},
  // interior faces first, then boundary faces), and per cell the face entries
  // of its edge slots (FR: four 16-bit refs, face << 1 | side, 0xFFFF none).
  const float4* FL = nullptr;
  const int32_t* FLoff = nullptr;
  const uint2* FR = nullptr;
  int32_t faceMax = 0;               // most faces in one tile
  // Kernel of the fused FP32 stages (hg_autotune): kStageGather, kStagePipe,
  // kStageTma (the same results) or kStageFace (each wet-wet face once); and
  // its shape: 0 the register budget of 4 resident blocks per SM, 1 of 3
  // (gather and face kernels; the arithmetic does not depend on it).
  int32_t stageKernel = 0;
  int32_t stageVariant = 0;
  const int32_t* bfInfo = nullptr;   // [nbf] type | group << 2
  const double* bfLp23 = nullptr;    // [nbf] L^(2/3) (inlet-Q faces)
  const double* bfLp53 = nullptr;    // [nbf] L^(5/3) (inlet-Q faces)
  const float* bfLp23f = nullptr;
  const float* bfExitRel = nullptr;  // [nbf] exit-H faces: (WSE - zb) - hstill of the face's cell, formed in FP64
  const int32_t* inletOff = nullptr; // [nInlet+1] CSR over inlet faces in NodeString order
  const int32_t* inletCell = nullptr;
  const double* inletLp53 = nullptr; // L^(5/3)
  // FP64 per-cell data
  const double* area = nullptr;
  const double* hst = nullptr;       // hstill
  const double* zb = nullptr;
  const double* man = nullptr;       // Manning n
  const double* s0x = nullptr;
  const double* s0y = nullptr;
  // FP32 per-cell data: CP {hstill_hi, hstill_lo, zb, n} (hstill as an exact
  // hi + lo pair), CS {S0x, S0y, area, 0}
  const float4* CP = nullptr;
  const float4* CS = nullptr;
  float hsmf = 1e-3f, gf = 9.81f, kn2f = 1.0f;
  float hsmLo = 0.0f;                // h_small - hsmf, so that hsmf + hsmLo is h_small to 2^-48
  // Boundary values
  const double* exitWse = nullptr;   // [nExit]
  const double* inletQ = nullptr;    // [nInlet]
  double* totalA = nullptr;          // [nInlet] conveyance of the current stage input
  // FP32 unfused conveyance totals (k_inlet_total_f32): each group's faces
  // split over inletParts blocks of kInletBlock, per-block partial sums and a
  // per-group arrival count.
  double* inletPart = nullptr;       // [nInlet][inletParts]
  unsigned int* inletTicket = nullptr;   // [nInlet], zero between launches
  int32_t inletParts = 1;
  double g = 9.81, kn2 = 1.0, hsm = 1e-3;
  ResDev res;
  // Inlet-Q hydrographs (hg_set_inlet_hydrograph): for each inlet-Q group g
  // with points, Q(t) interpolates (hydroT, hydroQ)[hydroOff[g] ..
  // hydroOff[g+1]) linearly (held at the end values outside them) and is
  // written into inletQ before each RHS evaluation (launch_hydrograph).
  int32_t nHydro = 0;                // points of all groups (0: constant discharges)
  const int32_t* hydroOff = nullptr; // [nInlet + 1]
  const double* hydroT = nullptr;
  const double* hydroQ = nullptr;
};

// Times at which launch_hydrograph evaluates the hydrographs.
enum HydroTime : int32_t {
  kHydroAt = 0,          // the time passed in
  kHydroStepStart = 1,   // the step begun by k_step_begin: elapsed time - dt
  kHydroStepEnd = 2,     // the elapsed time (stage 2 of SSP-RK2)
  kHydroNow = 3          // the elapsed time (fused stepping: before stage 1, t_n; before stage 2, t_n + dt)
};

// Scalars that live on the device so that steps can be captured in a graph.
struct DevScalars {
  double* dt = nullptr;                   // current step size
  float* dtf = nullptr;                   // the same, as float (FP32 path)
  unsigned long long* cflMin = nullptr;   // [2] min over cells of A / sum L(|u.n|+c), as ordered bits
  unsigned int* cflMinF = nullptr;        // [2] the same from the FP32 path (index 1: fused stepping only)
  double* dtHist = nullptr;               // [capacity] step sizes taken
  int32_t* stepIdx = nullptr;             // steps taken since the last reset
  double* tSum = nullptr;                 // sum of the steps taken
  int32_t* flags = nullptr;               // bit 0: non-finite state, bit 1: inlet conveyance <= 1e-10,
                                          // bit 3: a CFL step below dtMin
  int32_t dtCap = 0;
  double dtMin = 0.0;                     // smallest CFL step accepted (swe_2D_consts.dt_min)
  // Ensembles (nMembers > 0): every member takes its own step, as if it ran
  // alone.  Member m owns device cells [memberOff[m], memberOff[m + 1]); the
  // step bookkeeping forms each member's dt from its own CFL minimum (or the
  // fixed dt) into dtM / dtMf, the stage kernels read their cell's member's
  // step, and publish CFL candidates into the member's minimum.
  int32_t nMembers = 0;
  const int32_t* memberOff = nullptr;     // [nMembers + 1], device order
  const int32_t* memberOfCell = nullptr;  // [n] the member of each device cell
  const int32_t* inletMember = nullptr;   // [nInlet] member of each inlet-Q group (hydrograph times)
  double* dtM = nullptr;                  // [nMembers] current step
  float* dtMf = nullptr;
  double* tM = nullptr;                   // [nMembers] elapsed time
  unsigned long long* cflMinM = nullptr;  // [nMembers] CFL minimum, as ordered bits (FP64 path)
  unsigned int* cflMinMF = nullptr;       // [nMembers] the same (FP32 path)
  double* dtHistM = nullptr;              // [dtCap][nMembers] steps taken
};

// kModeRhsF32: the RHS as float (the FP32 stage kernel only; Rout then points
// at [3n] floats).
enum StageMode : int32_t { kModeRhs = 0, kModeStage1 = 1, kModeStage2 = 2, kModeEulerRef = 3, kModeRhsF32 = 4 };

// Fused FP32 stepping: one RK2 step is two launches.
//  * dt: in CFL mode thread 0 of every block forms dt = cfl * min from the
//    minimum the previous step published into cflMin[parity] / cflMinF[parity]
//    and shares it through shared memory; stage 2
//    publishes into the other buffer, and stage 1 of a step clears it (block 0),
//    which nobody reads during stage 1.  Stage 1's block 0 records the step.
//  * inlet-Q conveyance totals of a stage's output state (read by the next
//    stage's inlet ghosts): only the blocks holding inlet cells (blockSlot >= 0)
//    take part; each writes its partial sums, and the last of them to finish
//    (atomic ticket) adds them in slot order -- deterministic -- and resets the ticket.
constexpr int kMaxFusedInlets = 4;
struct StageFuse {
  const double* totalIn = nullptr;   // conveyance totals of the input state (replaces DevMesh::totalA)
  double* totalOut = nullptr;        // totals of the output state
  double* partials = nullptr;        // [kMaxFusedInlets][nSlots][kStageBlockF32 / 32] warp sums
  unsigned int* ticket = nullptr;
  const int32_t* blockSlot = nullptr;   // [tiles of kStageBlockF32 cells] slot of a tile holding inlet cells, else -1
  int32_t nSlots = 0;
  int32_t nWarps = 0;                // the warps of those tiles that hold cells (arrivals before the last)
  int32_t record = 0;                // stage 1: block 0 records the step and clears the other CFL buffer
  int32_t cflMode = 0;
  int32_t parity = 0;
  double cfl = 0.0;
};

// FP64 state: Q blocks [xi | qx | qy] of n doubles.
void launch_inlet_total_f64(const DevMesh& m, const DevScalars& s, const double* Q, cudaStream_t st);
void launch_stage_f64(const DevMesh& m, const DevScalars& s, int mode, const double* Qin, const double* Qbase,
                      double* Qout, bool cfl, cudaStream_t st);
void launch_cfl_f64(const DevMesh& m, const DevScalars& s, const double* Q, cudaStream_t st);

// FP32-compensated state: x[c] {xi_hi, xi_lo, qx_hi, qy_hi}, q[c] {qx_lo, qy_lo}.
struct StateF32 {
  float4* x = nullptr;
  float2* q = nullptr;
};
void launch_inlet_total_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st);
// Resistance of the state (see ResDev); the number of launches it makes.
// launch_inlet_total_f64 / _f32 call these first, so every RHS evaluation sees
// the resistance of its own input state.
int launch_resistance_f64(const DevMesh& m, const double* Q, cudaStream_t st);
// inletQ[g] = Q_g(t) for every inlet-Q group with a hydrograph (a no-op
// without one); the number of launches it made.
int launch_hydrograph(const DevMesh& m, const DevScalars& s, int when, double t, cudaStream_t st);
int launch_resistance_f32(const DevMesh& m, StateF32 X, cudaStream_t st);
int resistance_launches(const DevMesh& m);
void launch_stage_f32(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                      double* Rout, bool cfl, cudaStream_t st);
// Stage with the fused work of StageFuse (requires nInlet <= kMaxFusedInlets).
void launch_stage_f32_fused(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase,
                            StateF32 Xout, const StageFuse& f, cudaStream_t st);
// Blocks of an FP32 stage launch; block b holds cells [b * kStageBlockF32, (b + 1) * kStageBlockF32).
#ifndef HG_STAGE_BLOCK
#define HG_STAGE_BLOCK 256
#endif
constexpr int kStageBlockF32 = HG_STAGE_BLOCK;
constexpr int kHaloMax = 128;   // out-of-tile neighbour cells a pipelined stage tile can hold
enum StageKernel : int32_t { kStageGather = 0, kStagePipe = 1, kStageTma = 2, kStageFace = 3 };
// Packed ids of a face-once face record (FL .w as int bits): interior faces
// a | b << 10 | a-in-tile << 20 | b-in-tile << 21 (tile-local indices: own
// cells [0, kStageBlockF32), halo cells kStageBlockF32 + j); boundary faces
// a | bf << 10 | 1 << 31 (bf < 2^21).
constexpr int32_t kFaceBoundary = INT32_MIN;
constexpr int kFaceMaxPerTile = 1024;
int stage_blocks_f32(const DevMesh& m);
// The kernel HG_STAGE_KERNEL forces (gather / pipe / tma / face), else -1;
// the shape HG_STAGE_VARIANT forces (0 to 3), else -1.
int stage_kernel_forced();
int stage_variant_forced();
// Whether kernel k can run the fused stages of this mesh and these states.
bool stage_kernel_usable(const DevMesh& m, int k, int mode, StateF32 Xin, StateF32 Xbase);
// Clear CFL-minimum buffer `parity` (fused stepping keeps two).
void launch_reset_cfl(const DevScalars& s, int parity, cudaStream_t st);
void launch_cfl_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st);

// Step bookkeeping: when cflMode, dt = cfl * min; records dt and resets the min.
void launch_step_begin(const DevScalars& s, bool cflMode, double cfl, cudaStream_t st);
void launch_reset_scalars(const DevScalars& s, cudaStream_t st);

// Renumbering between the caller's order (user) and the device order.
void launch_gather_state_f64(int32_t n, const int32_t* perm, const double* user, double* dev, cudaStream_t st);
// Block size of per-cell FP64 kernels on an n-cell mesh (256, smaller on small meshes).
int stage_block_f64(int n);
void launch_scatter_state_f64(int32_t n, const int32_t* perm, const double* dev, double* user, cudaStream_t st);
void launch_scatter_field_f64(int32_t n, const int32_t* perm, const double* dev, const double* add, double* user,
                              cudaStream_t st);
void launch_gather_state_f32(int32_t n, const int32_t* perm, const double* user, StateF32 dev, cudaStream_t st);
void launch_scatter_state_f32(int32_t n, const int32_t* perm, StateF32 dev, double* user, cudaStream_t st);
// L2 flush over a buffer of `bytes` (> 2x L2): returns the launches made.
int launch_flush(void* buf, size_t bytes, cudaStream_t st);

}  // namespace hg
