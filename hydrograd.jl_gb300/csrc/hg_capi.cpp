// C ABI implementation: context lifecycle, parameter upload, host<->device
// state transfer, and the step sequences (graph-captured on request).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hg_adjoint.hpp"
#include "hg_autotune.hpp"
#include "hg_ctx.hpp"
#include "hg_mesh.hpp"
#include "hg_state.hpp"
#include "hydrograd_gb.h"

using namespace hg;

namespace {

thread_local std::string g_err;

// Smallest CFL step accepted by default: swe_2D_consts.dt_min, which the
// reference sets to 0.001 s (solve_swe_2D.jl:83,98) and stores unused.
constexpr double kDtMinDefault = 0.001;
// Stage-kernel family of a new context (hg_set_stage_family): 0 gather.  On
// the 1M-cell reach the face-once kernel ties the gather kernel on stage 1
// (37.0 against 36.0 us) and loses on stage 2, so it is the opt-in family.
constexpr int kDefaultFamily = 0;

int fail(hg_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  else g_err = msg;
  return code;
}

#define HG_CUDA(ctx, call)                                                                        \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail((ctx), HG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));        \
  } while (0)

template <class T>
cudaError_t dalloc(hg_ctx* c, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
  if (e == cudaSuccess) {
    c->allocs.push_back(q);
    *p = static_cast<T*>(q);
  }
  return e;
}

template <class T>
cudaError_t upload(hg_ctx* c, T* d, const std::vector<T>& h) {
  if (h.empty()) return cudaSuccess;
  return cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream);
}

std::vector<float> to_float(const std::vector<double>& v) {
  std::vector<float> r(v.size());
  for (size_t i = 0; i < v.size(); ++i) r[i] = (float)v[i];
  return r;
}

// Bed data from zb at cells (process_bed_2D.jl:46-66; fvm_schemes_2D.jl:197-213,253-275),
// in the reference's operation order.  Outputs in the caller's cell order.
void compute_bed(const HostMesh& m, const std::vector<double>& zb, std::vector<double>& s0x, std::vector<double>& s0y) {
  std::vector<double> zf(m.nFaces);
  for (int f = 0; f < m.nFaces; ++f)
    zf[f] = m.faceC1[f] >= 0 ? (zb[m.faceC0[f]] + zb[m.faceC1[f]]) / 2.0 : zb[m.faceC0[f]];
  s0x.assign(m.nCells, 0.0);
  s0y.assign(m.nCells, 0.0);
  for (int c = 0; c < m.nCells; ++c) {
    double gx = 0.0, gy = 0.0;
    for (int i = 0; i < m.ncf[c]; ++i) {
      const int f = m.cf[(size_t)c * 8 + i];
      gx = gx + m.snx[(size_t)c * 8 + i] * zf[f] * m.faceLen[f];
      gy = gy + m.sny[(size_t)c * 8 + i] * zf[f] * m.faceLen[f];
    }
    s0x[c] = -1.0 * (gx / m.area[c]);
    s0y[c] = -1.0 * (gy / m.area[c]);
  }
}

template <class T>
std::vector<T> to_device_order(const hg_ctx* c, const T* user) {
  std::vector<T> r(c->n);
  for (int i = 0; i < c->n; ++i) r[i] = user[c->perm[i]];
  return r;
}

// The FP32 path's exit-H surface offset xi_ghost = (WSE - zb) - hstill per
// exit face, in FP64 (bc_2D.jl exit-H ghost depth; hstill as the RHS sees it).
// Formed in FP32 from a rounded WSE and zb it would carry an error of a few
// 1e-7 m, which the Roe dissipation turns into a spurious outflow.
int upload_exit_rel(hg_ctx* c) {
  if (!c->d_bfExitRel) return HG_OK;
  for (size_t e = 0; e < c->exitBf.size(); ++e) {
    const int cell = c->exitCell[e];
    c->h_bfExitRel[c->exitBf[e]] = (float)((c->exitWse[c->exitGrp[e]] - c->zbCell[cell]) - c->hstill[cell]);
  }
  HG_CUDA(c, upload(c, c->d_bfExitRel, c->h_bfExitRel));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  return HG_OK;
}

int upload_cells(hg_ctx* c) {
  // FP64 and FP32 copies of the per-cell parameters, in device order.
  std::vector<double> hst = to_device_order(c, c->hstill.data());
  std::vector<double> zb = to_device_order(c, c->zbCell.data());
  std::vector<double> man = to_device_order(c, c->manning.data());
  std::vector<double> s0x = to_device_order(c, c->s0x.data());
  std::vector<double> s0y = to_device_order(c, c->s0y.data());
  HG_CUDA(c, upload(c, c->d_hst, hst));
  HG_CUDA(c, upload(c, c->d_zb, zb));
  HG_CUDA(c, upload(c, c->d_man, man));
  HG_CUDA(c, upload(c, c->d_s0x, s0x));
  HG_CUDA(c, upload(c, c->d_s0y, s0y));
  // FP32 records: CP {hstill_hi, hstill_lo, zb, n}, CS {S0x, S0y, area, 0}.
  c->h_CP.resize(c->n);
  c->h_CS.resize(c->n);
  for (int i = 0; i < c->n; ++i) {
    const float hh = (float)hst[i];
    c->h_CP[i] = make_float4(hh, (float)(hst[i] - (double)hh), (float)zb[i], (float)man[i]);
    c->h_CS[i] = make_float4((float)s0x[i], (float)s0y[i], c->h_area[i], 0.0f);
  }
  HG_CUDA(c, upload(c, c->d_CP, c->h_CP));
  HG_CUDA(c, upload(c, c->d_CS, c->h_CS));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  return upload_exit_rel(c);
}

int upload_boundary_values(hg_ctx* c) {
  HG_CUDA(c, upload(c, c->d_inletQ, c->inletQ));
  HG_CUDA(c, upload(c, c->d_exitWse, c->exitWse));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  return upload_exit_rel(c);
}

int check_flags(hg_ctx* c) {
  int32_t f = 0;
  HG_CUDA(c, cudaMemcpyAsync(&f, c->ds.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (f & 2) return fail(c, HG_ERR_INLET, "inlet-Q total conveyance is not positive (all inlet cells dry?)");
  if (f & 1) return fail(c, HG_ERR_STATE, "non-finite value in the state");
  if (f & 8)
    return fail(c, HG_ERR_STATE, "the CFL time step fell below dt_min (" + std::to_string(c->ds.dtMin) +
                                     " s; hg_set_dt_min): the state is collapsing");
  return HG_OK;
}

int ensure_dt_capacity(hg_ctx* c, int32_t steps) {
  if (steps <= c->ds.dtCap) return HG_OK;
  int32_t cap = std::max(steps, 2 * c->ds.dtCap);
  double* p = nullptr;
  HG_CUDA(c, cudaMalloc(&p, (size_t)cap * sizeof(double)));
  if (c->ds.dtHist) cudaFree(c->ds.dtHist);
  c->ds.dtHist = p;
  if (c->ds.nMembers > 0) {   // each member's steps: [cap][members]
    double* pm = nullptr;
    HG_CUDA(c, cudaMalloc(&pm, (size_t)cap * c->ds.nMembers * sizeof(double)));
    if (c->ds.dtHistM) cudaFree(c->ds.dtHistM);
    c->ds.dtHistM = pm;
  }
  c->ds.dtCap = cap;
  c->graphValid = false;   // the captured scalars struct holds the old pointer
  return HG_OK;
}

StateF32 xa(hg_ctx* c) { return StateF32{c->XA, c->XQA}; }
StateF32 xb(hg_ctx* c) { return StateF32{c->XB, c->XQB}; }

// Enqueue the state upload from a host buffer (caller order).
int enqueue_upload(hg_ctx* c, const double* Q) {
  HG_CUDA(c, cudaMemcpyAsync(c->Quser, Q, (size_t)3 * c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->precision == HG_FP64) launch_gather_state_f64(c->n, c->d_perm, c->Quser, c->QA, c->stream);
  else launch_gather_state_f32(c->n, c->d_perm, c->Quser, xa(c), c->stream);
  c->launches += 1;
  return HG_OK;
}

int enqueue_download(hg_ctx* c, double* Q) {
  if (c->precision == HG_FP64) launch_scatter_state_f64(c->n, c->d_perm, c->QA, c->Quser, c->stream);
  else launch_scatter_state_f32(c->n, c->d_perm, xa(c), c->Quser, c->stream);
  c->launches += 1;
  HG_CUDA(c, cudaMemcpyAsync(Q, c->Quser, (size_t)3 * c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return HG_OK;
}

// The FP32 path steps with two fused launches when the inlet groups fit and
// the resistance does not depend on the state (the fused stage forms the next
// stage's conveyance totals from its output state with the resident n).
// Fused FP32C steps: constant n, or n from an n(h, Umag, ks) function of the
// state, which the fused kernels evaluate themselves (not the UDE closures,
// whose LayerNorm statistics span all cells).
bool fused(const hg_ctx* c) {
  const int32_t k = c->dm.res.kind;
  return c->precision == HG_FP32C && c->dm.nInlet <= kMaxFusedInlets &&
         (k == kResConstant || (k >= kResPowerLaw && k <= kResHUmagKs)) && c->ds.nMembers == 0;
}

// Kernels per RHS evaluation besides the stage: resistance, inlet totals.
int rhs_prep_launches(const hg_ctx* c) { return resistance_launches(c->dm) + (c->dm.nInlet > 0 ? 1 : 0); }

// Before a run of fused steps: conveyance totals of the resident state and, in
// CFL mode, its CFL minimum in buffer 0 (the fixed dt is already on the device).
void enqueue_fused_prime(hg_ctx* c, bool cflMode) {
  DevMesh m = c->dm;
  m.totalA = c->d_tot;
  launch_inlet_total_f32(m, c->ds, xa(c), c->stream);
  c->parity = 0;
  if (cflMode) {
    launch_reset_cfl(c->ds, 0, c->stream);
    launch_cfl_f32(c->dm, c->ds, xa(c), c->stream);
  }
  c->launches += (c->dm.nInlet > 0 ? 1 : 0) + (cflMode ? 2 : 0);
}

// One fused SSP-RK2 step: stage 1 (records the step, totals of Q1), stage 2
// (totals of Q2 and the CFL minimum of Q2 for the next step).
void enqueue_rk2_step_fused(hg_ctx* c, bool cflMode, double cfl) {
  StageFuse f;
  f.partials = c->d_partials;
  f.ticket = c->d_ticket;
  f.blockSlot = c->d_blockSlot;
  f.nSlots = c->nSlots;
  f.nWarps = c->nWarps;
  f.cflMode = cflMode ? 1 : 0;
  f.cfl = cfl;
  f.parity = c->parity;
  f.record = 1;
  f.totalIn = c->d_tot;
  f.totalOut = c->d_tot + kMaxFusedInlets;
  // inlet hydrographs: t_n before stage 1, t_n + dt (recorded by stage 1) before stage 2
  const int hyd = launch_hydrograph(c->dm, c->ds, kHydroNow, 0.0, c->stream);
  launch_stage_f32_fused(c->dm, c->ds, kModeStage1, xa(c), StateF32{}, xb(c), f, c->stream);
  f.record = 0;
  f.totalIn = c->d_tot + kMaxFusedInlets;
  f.totalOut = c->d_tot;
  launch_hydrograph(c->dm, c->ds, kHydroNow, 0.0, c->stream);
  launch_stage_f32_fused(c->dm, c->ds, kModeStage2, xb(c), xa(c), xa(c), f, c->stream);
  c->parity ^= 1;
  c->launches += 2 + 2 * hyd;
}

// One SSP-RK2 step on the resident state (QA / XA).  Unfused kernels per step:
// step_begin, [inlet], stage1, [inlet], stage2.
void enqueue_rk2_step(hg_ctx* c, bool cflMode, double cfl) {
  if (fused(c)) {
    enqueue_rk2_step_fused(c, cflMode, cfl);
    return;
  }
  launch_step_begin(c->ds, cflMode, cfl, c->stream);
  // inlet hydrographs at each stage's time: t_n, then t_n + dt
  const int hyd = launch_hydrograph(c->dm, c->ds, kHydroStepStart, 0.0, c->stream);
  if (c->precision == HG_FP64) {
    launch_inlet_total_f64(c->dm, c->ds, c->QA, c->stream);
    launch_stage_f64(c->dm, c->ds, kModeStage1, c->QA, nullptr, c->QB, false, c->stream);
    launch_hydrograph(c->dm, c->ds, kHydroStepEnd, 0.0, c->stream);
    launch_inlet_total_f64(c->dm, c->ds, c->QB, c->stream);
    launch_stage_f64(c->dm, c->ds, kModeStage2, c->QB, c->QA, c->QA, cflMode, c->stream);
  } else {
    launch_inlet_total_f32(c->dm, c->ds, xa(c), c->stream);
    launch_stage_f32(c->dm, c->ds, kModeStage1, xa(c), StateF32{}, xb(c), nullptr, false, c->stream);
    launch_hydrograph(c->dm, c->ds, kHydroStepEnd, 0.0, c->stream);
    launch_inlet_total_f32(c->dm, c->ds, xb(c), c->stream);
    launch_stage_f32(c->dm, c->ds, kModeStage2, xb(c), xa(c), xa(c), nullptr, cflMode, c->stream);
  }
  c->launches += 3 + 2 * rhs_prep_launches(c) + 2 * hyd;
}

void enqueue_euler_step(hg_ctx* c, bool cflMode, double cfl) {
  launch_step_begin(c->ds, cflMode, cfl, c->stream);
  c->launches += launch_hydrograph(c->dm, c->ds, kHydroStepStart, 0.0, c->stream);
  if (c->precision == HG_FP64) {
    launch_inlet_total_f64(c->dm, c->ds, c->QA, c->stream);
    launch_stage_f64(c->dm, c->ds, kModeEulerRef, c->QA, nullptr, c->QB, false, c->stream);
    if (cflMode) launch_cfl_f64(c->dm, c->ds, c->QB, c->stream);
    std::swap(c->QA, c->QB);
  } else {
    launch_inlet_total_f32(c->dm, c->ds, xa(c), c->stream);
    launch_stage_f32(c->dm, c->ds, kModeEulerRef, xa(c), StateF32{}, xb(c), nullptr, false, c->stream);
    if (cflMode) launch_cfl_f32(c->dm, c->ds, xb(c), c->stream);
    std::swap(c->XA, c->XB);
    std::swap(c->XQA, c->XQB);
  }
  c->launches += 2 + rhs_prep_launches(c) + (cflMode ? 1 : 0);
}

void enqueue_cfl_prime(hg_ctx* c) {
  if (c->precision == HG_FP64) launch_cfl_f64(c->dm, c->ds, c->QA, c->stream);
  else launch_cfl_f32(c->dm, c->ds, xa(c), c->stream);
  c->launches += 1;
}

int set_fixed_dt(hg_ctx* c, double dt) {
  float dtf = (float)dt;
  HG_CUDA(c, cudaMemcpyAsync(c->ds.dt, &dt, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  HG_CUDA(c, cudaMemcpyAsync(c->ds.dtf, &dtf, sizeof(float), cudaMemcpyHostToDevice, c->stream));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  return HG_OK;
}

// Autotuner of the fused FP32 stages.  Its candidates are kernels and shapes
// that compute bit-identical results, so the choice changes speed only:
//   family 0: the gather kernel in four shapes -- 256-cell blocks with the
//             register budget of 4 or 3 resident per SM, 512-cell blocks at
//             2 per SM, 128-cell blocks at 8 per SM -- the pipelined
//             persistent kernel, the bulk-copy persistent kernel;
//   family 1: the face-once kernel with the budget of 4 or 3 blocks per SM.
// (The face-once kernel evaluates each wet-wet face once and so rounds
// differently from the gather family; which family a context uses is fixed by
// hg_set_stage_family / HG_STAGE_FAMILY, never by timing.)  The usable
// candidates are timed on the resident state, a stage-1 and a stage-2 launch
// per repetition, each repetition after an L2 flush and the candidates
// interleaved; the fastest is kept and written to the cache file
// (hg_autotune.hpp) under a key of the GPU, the mesh's face tables, the
// precision, the Riemann solver and the family, so a later context on the
// same mesh and GPU takes it without timing.  Outputs go to scratch carved from
// the flush buffer (the flush overwrites it before the next repetition's
// stage 1 writes it again); the resident state, the step bookkeeping and the
// error flags are left as they were.
std::vector<TuneChoice> stage_candidates(const hg_ctx* c, StateF32 s1) {
  std::vector<TuneChoice> all;
  if (c->stageFamily == 1) {
    all = {TuneChoice{kStageFace, 0}, TuneChoice{kStageFace, 1}};
  } else {
    all = {TuneChoice{kStageGather, 0}, TuneChoice{kStageGather, 1}, TuneChoice{kStageGather, 2},
           TuneChoice{kStageGather, 3}, TuneChoice{kStagePipe, 0}, TuneChoice{kStageTma, 0}};
    if (c->dm.nslot > 4) all = {TuneChoice{kStageGather, 0}};
  }
  std::vector<TuneChoice> out;
  for (const TuneChoice& t : all)
    if (stage_kernel_usable(c->dm, t.kernel, kModeStage1, StateF32{c->XA, c->XQA}, StateF32{}) &&
        stage_kernel_usable(c->dm, t.kernel, kModeStage2, s1, StateF32{c->XA, c->XQA}))
      out.push_back(t);
  return out;
}

std::string autotune_key(const hg_ctx* c) {
  cudaDeviceProp p{};
  cudaGetDeviceProperties(&p, c->device);
  char sig[32];
  std::snprintf(sig, sizeof(sig), "%016llx", (unsigned long long)c->meshSig);
  return std::string(p.name) + "|sm" + std::to_string(p.major * 10 + p.minor) + "|fp32c|family" +
         std::to_string(c->stageFamily) + "|rs" + std::to_string(c->dm.riemann) + "|n" + std::to_string(c->n) +
         "|s" + std::to_string(c->dm.nslot) + "|" + sig;
}

void set_stage_choice(hg_ctx* c, const TuneChoice& t) {
  if (c->dm.stageKernel != t.kernel || c->dm.stageVariant != t.variant) c->graphValid = false;
  c->dm.stageKernel = t.kernel;
  c->dm.stageVariant = t.variant;
}

// useCache: take a cached choice instead of timing (the automatic tune of a
// context's first steps); an explicit hg_autotune times and rewrites it.
int autotune_stage(hg_ctx* c, int reps, bool useCache) {
  if (!fused(c) || c->dm.res.kind != kResConstant) return HG_OK;   // (n functions: one fixed kernel)
  const size_t n = (size_t)c->n;
  const size_t rec = (n * sizeof(float4) + 255) & ~(size_t)255, lo = (n * sizeof(float2) + 255) & ~(size_t)255;
  if (2 * (rec + lo) > c->flushBytes) return HG_OK;   // no scratch: keep the default
  char* base = static_cast<char*>(c->flushBuf);
  const StateF32 s1{reinterpret_cast<float4*>(base), reinterpret_cast<float2*>(base + rec)};
  const StateF32 s2{reinterpret_cast<float4*>(base + rec + lo), reinterpret_cast<float2*>(base + 2 * rec + lo)};
  const std::vector<TuneChoice> cand = stage_candidates(c, s1);
  if (cand.empty()) return HG_OK;
  const std::string path = autotune_cache_path();
  const std::string key = autotune_key(c);
  if (useCache) {
    TuneChoice t;
    if (autotune_cache_load(path, key, t))
      for (const TuneChoice& x : cand)
        if (x.kernel == t.kernel && x.variant == t.variant) {
          set_stage_choice(c, t);
          c->stageTuned = true;
          c->tuneSource = 2;
          return HG_OK;
        }
  }
  int32_t flags = 0;
  HG_CUDA(c, cudaMemcpyAsync(&flags, c->ds.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  std::vector<double> total(cand.size(), 0.0);
  cudaEvent_t a, b;
  HG_CUDA(c, cudaEventCreate(&a));
  HG_CUDA(c, cudaEventCreate(&b));
  StageFuse f;   // fixed dt, no step record, totals into the stage buffer's slots
  f.partials = c->d_partials;
  f.ticket = c->d_ticket;
  f.blockSlot = c->d_blockSlot;
  f.nSlots = c->nSlots;
  f.nWarps = c->nWarps;
  for (int r = 0; r < reps; ++r)
    for (size_t i = 0; i < cand.size(); ++i) {
      DevMesh m = c->dm;
      m.stageKernel = cand[i].kernel;
      m.stageVariant = cand[i].variant;
      c->launches += launch_flush(c->flushBuf, c->flushBytes, c->stream);
      cudaEventRecord(a, c->stream);
      f.totalIn = c->d_tot;
      f.totalOut = c->d_tot + kMaxFusedInlets;
      launch_stage_f32_fused(m, c->ds, kModeStage1, xa(c), StateF32{}, s1, f, c->stream);
      f.totalIn = c->d_tot + kMaxFusedInlets;
      launch_stage_f32_fused(m, c->ds, kModeStage2, s1, xa(c), s2, f, c->stream);
      cudaEventRecord(b, c->stream);
      cudaEventSynchronize(b);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      total[i] += ms;
      c->launches += 2;
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  HG_CUDA(c, cudaGetLastError());
  HG_CUDA(c, cudaMemcpyAsync(c->ds.flags, &flags, sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  size_t best = 0;
  for (size_t i = 1; i < cand.size(); ++i)
    if (total[i] < total[best]) best = i;
  set_stage_choice(c, cand[best]);
  c->stageTuned = true;
  c->tuneSource = 1;
  if (reps > 0) autotune_cache_store(path, key, cand[best], total[best] / reps);
  return HG_OK;
}

// Set-up before a run of RK2 steps (rk2 = false: reference Euler steps).
int begin_steps(hg_ctx* c, bool rk2, double dt, double cfl) {
  const bool cflMode = dt <= 0;
  if (!cflMode) {
    int rc = set_fixed_dt(c, dt);
    if (rc) return rc;
  }
  if (rk2 && fused(c) && !c->stageTuned && stage_kernel_forced() < 0) {
    int rc = autotune_stage(c, 3, true);
    if (rc) return rc;
  }
  if (rk2 && fused(c)) {
    enqueue_fused_prime(c, cflMode);
  } else if (cflMode && !c->cflPrimed) {
    enqueue_cfl_prime(c);
  }
  return HG_OK;
}

// Network parameters a hg_ude_desc can describe (3 inputs, 4 hidden layers of 16).
constexpr int kResMaxParams = kResMaxInputs * kResMaxWidth + 3 * kResMaxWidth +
                              (kResMaxLayers - 1) * (kResMaxWidth * kResMaxWidth + 3 * kResMaxWidth) +
                              kResMaxWidth + 1;

// Puts r in place as the context's resistance: device buffers on first use,
// ks and the network parameters uploaded, the captured graph dropped (it holds
// the old DevMesh by value).
int install_resistance(hg_ctx* c, ResDev r, const double* ksUser, const double* params, int nParams) {
  if (!c->d_resKs) {
    HG_CUDA(c, dalloc(c, &c->d_resKs, c->n));
    HG_CUDA(c, dalloc(c, &c->d_resW, kResMaxParams));
    HG_CUDA(c, dalloc(c, &c->d_resWf, kResMaxParams));
    HG_CUDA(c, dalloc(c, &c->d_resStats, 2 * kResMaxLayers));
    HG_CUDA(c, dalloc(c, &c->d_resPartials, 4 * (size_t)res_stat_blocks(c->n)));
    HG_CUDA(c, dalloc(c, &c->d_resTicket, 1));
    HG_CUDA(c, dalloc(c, &c->d_fres, c->n));
    HG_CUDA(c, dalloc(c, &c->d_fresF, c->n));
    HG_CUDA(c, cudaMemsetAsync(c->d_resTicket, 0, sizeof(unsigned int), c->stream));
  }
  std::vector<double> ks, w(params, params + nParams);
  std::vector<float> wf = to_float(w);
  if (ksUser) ks = to_device_order(c, ksUser);
  HG_CUDA(c, upload(c, c->d_resKs, ks));
  HG_CUDA(c, upload(c, c->d_resW, w));
  HG_CUDA(c, upload(c, c->d_resWf, wf));
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  r.ks = ksUser ? c->d_resKs : nullptr;
  r.w = c->d_resW;
  r.wf = c->d_resWf;
  r.stats = c->d_resStats;
  r.partials = c->d_resPartials;
  r.ticket = c->d_resTicket;
  r.fres = c->d_fres;
  r.fresF = c->d_fresF;
  if (r.kind >= kResUdeManningH && r.overBatch && r.nHidden > 0) {   // the statistics passes' cache of the hidden layers
    size_t rows = 0;
    for (int l = 0; l < r.nHidden; ++l) rows += (size_t)r.width[l];
    const size_t bytes = rows * (size_t)c->n * (c->precision == HG_FP64 ? sizeof(double) : sizeof(float));
    if (bytes > c->resActBytes) {
      cudaFree(c->d_resAct);
      c->d_resAct = nullptr;
      c->resActBytes = 0;
      HG_CUDA(c, cudaMalloc(&c->d_resAct, bytes));
      c->resActBytes = bytes;
    }
    if (c->precision == HG_FP64) r.hid = static_cast<double*>(c->d_resAct);
    else r.hidF = static_cast<float*>(c->d_resAct);
  }
  c->dm.res = r;
  c->udeParams = r.kind >= kResUdeManningH ? nParams : 0;
  c->udeGrad.clear();
  c->graphValid = false;
  return HG_OK;
}

// Face-once stage tables (k_stage_face_f32): per tile of kStageBlockF32 cells
// its faces, each listed once -- interior faces (both cells in the tile, or
// one a halo cell) oriented from the lower cell id and in the order their
// lower cell meets them, then the tile's boundary faces -- and per cell the
// entry (face << 1 | side) of each edge slot.  SLp holds the pipelined
// kernel's tile-local neighbour indices (halo cells kStageBlockF32 + j).
// False when the tables do not fit their encodings: a tile with more than
// kFaceMaxPerTile faces, a boundary-face index of more than 21 bits, or an
// interior face that only one of its cells lists.
bool build_face_tables(int N, int S, int nbf, const std::vector<int32_t>& nb, const std::vector<float4>& SL,
                       const std::vector<float4>& SLp, std::vector<float4>& FL, std::vector<int32_t>& FLoff,
                       std::vector<uint2>& FR, int32_t& faceMax) {
  if (S > 4 || nbf >= (1 << 21) || SLp.size() != (size_t)S * N) return false;
  const int nTiles = (N + kStageBlockF32 - 1) / kStageBlockF32;
  FL.clear();
  FLoff.assign((size_t)nTiles + 1, 0);
  faceMax = 0;
  std::vector<uint16_t> ref((size_t)N * 4, 0xFFFFu);
  auto back_slot = [&](int v, int cell) {
    for (int k = 0; k < S; ++k)
      if (nb[(size_t)k * N + v] == cell) return k;
    return -1;
  };
  auto with_ids = [](float4 r, int32_t w) {
    std::memcpy(&r.w, &w, sizeof(float));
    return r;
  };
  std::vector<float4> inner, bnd;
  std::vector<size_t> bndRef;
  for (int t = 0; t < nTiles; ++t) {
    const int c0 = t * kStageBlockF32, c1 = std::min(N, c0 + kStageBlockF32);
    inner.clear();
    bnd.clear();
    bndRef.clear();
    for (int cell = c0; cell < c1; ++cell)
      for (int k = 0; k < S; ++k) {
        const size_t i = (size_t)k * N + cell;
        const int32_t v = nb[i];
        if (v == INT32_MIN) continue;
        const int32_t la = cell - c0;
        if (v < 0) {   // boundary face -1 - v
          bnd.push_back(with_ids(SL[i], la | ((-1 - v) << 10) | kFaceBoundary));
          bndRef.push_back((size_t)cell * 4 + k);
          continue;
        }
        if (v >= c0 && v < c1) {   // both cells in the tile: listed once, by the lower id
          if (v < cell) continue;
          const int kb = back_slot(v, cell);
          if (kb < 0) return false;
          const uint16_t f = (uint16_t)inner.size();
          inner.push_back(with_ids(SL[i], la | ((v - c0) << 10) | (1 << 20) | (1 << 21)));
          ref[(size_t)cell * 4 + k] = (uint16_t)(f << 1);
          ref[(size_t)v * 4 + kb] = (uint16_t)((f << 1) | 1);
          continue;
        }
        int32_t lh;   // v's tile-local halo index
        std::memcpy(&lh, &SLp[i].w, sizeof(int32_t));
        const uint16_t f = (uint16_t)inner.size();
        if (cell < v) {   // oriented from the own cell (side a)
          inner.push_back(with_ids(SL[i], la | (lh << 10) | (1 << 20)));
          ref[(size_t)cell * 4 + k] = (uint16_t)(f << 1);
        } else {          // oriented from the halo cell: its slot's normal; the own cell is side b
          const int kb = back_slot(v, cell);
          if (kb < 0) return false;
          inner.push_back(with_ids(SL[(size_t)kb * N + v], lh | (la << 10) | (1 << 21)));
          ref[(size_t)cell * 4 + k] = (uint16_t)((f << 1) | 1);
        }
      }
    const size_t nF = inner.size() + bnd.size();
    if (nF > (size_t)kFaceMaxPerTile) return false;
    faceMax = std::max(faceMax, (int32_t)nF);
    for (size_t j = 0; j < bnd.size(); ++j) ref[bndRef[j]] = (uint16_t)((inner.size() + j) << 1);
    FL.insert(FL.end(), inner.begin(), inner.end());
    FL.insert(FL.end(), bnd.begin(), bnd.end());
    FLoff[(size_t)t + 1] = (int32_t)FL.size();
  }
  FR.resize(N);
  for (int c = 0; c < N; ++c) {
    const uint16_t* r = &ref[(size_t)c * 4];
    FR[c] = make_uint2((uint32_t)r[0] | ((uint32_t)r[1] << 16), (uint32_t)r[2] | ((uint32_t)r[3] << 16));
  }
  return true;
}

bool all_positive(const double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (!(v[i] > 0.0)) return false;
  return true;
}

}  // namespace

hg_ctx::~hg_ctx() {
  if (graphExec) cudaGraphExecDestroy(graphExec);
  if (stream) cudaStreamSynchronize(stream);
  for (void* p : allocs) cudaFree(p);
  if (ds.dtHist) cudaFree(ds.dtHist);
  if (ds.dtHistM) cudaFree(ds.dtHistM);
  if (d_resAct) cudaFree(d_resAct);
  adjoint_release(this);
  if (stream) cudaStreamDestroy(stream);
}

extern "C" {

int hg_abi_version(void) { return HG_ABI_VERSION; }

int hg_last_error(const hg_ctx* ctx, char* buf, int32_t len) {
  if (!buf || len <= 0) return HG_ERR_ARG;
  const std::string& s = ctx ? ctx->err : g_err;
  std::snprintf(buf, (size_t)len, "%s", s.c_str());
  return HG_OK;
}

int hg_mesh_build(const hg_mesh_desc* desc, hg_mesh** out) {
  if (!desc || !out) return fail(nullptr, HG_ERR_ARG, "hg_mesh_build: null argument");
  *out = nullptr;
  try {
    auto m = std::make_unique<hg_mesh>();
    std::string err;
    int rc = build_host_mesh(*desc, m->m, err);
    if (rc != HG_OK) return fail(nullptr, rc, err);
    *out = m.release();
    return HG_OK;
  } catch (const std::bad_alloc&) {
    return fail(nullptr, HG_ERR_ARG, "hg_mesh_build: out of host memory");
  }
}

int hg_mesh_free(hg_mesh* mesh) {
  delete mesh;
  return HG_OK;
}

static int sizes_of(const HostMesh& m, int32_t* s) {
  s[0] = m.nCells; s[1] = m.nFaces; s[2] = m.nGhost;
  s[3] = (int32_t)m.inletGroups.size(); s[4] = (int32_t)m.exitGroups.size();
  s[5] = (int32_t)m.wallGroups.size(); s[6] = (int32_t)m.symmGroups.size();
  s[7] = m.maxCellFaces;
  return HG_OK;
}

int hg_mesh_sizes(const hg_mesh* mesh, int32_t* sizes8) {
  if (!mesh || !sizes8) return fail(nullptr, HG_ERR_ARG, "hg_mesh_sizes: null argument");
  return sizes_of(mesh->m, sizes8);
}

int hg_mesh_cell_faces(const hg_mesh* mesh, int32_t* nbr8, double* normals16, double* lengths8, double* areas,
                       double* centroids2) {
  if (!mesh) return fail(nullptr, HG_ERR_ARG, "hg_mesh_cell_faces: null mesh");
  const HostMesh& m = mesh->m;
  for (int c = 0; c < m.nCells; ++c) {
    for (int i = 0; i < 8; ++i) {
      const bool has = i < m.ncf[c];
      const size_t k = (size_t)c * 8 + i;
      if (nbr8) nbr8[k] = has ? m.nbr[k] : -2;
      if (normals16) {
        normals16[2 * k] = has ? m.snx[k] : 0.0;
        normals16[2 * k + 1] = has ? m.sny[k] : 0.0;
      }
      if (lengths8) lengths8[k] = has ? m.faceLen[m.cf[k]] : 0.0;
    }
    if (areas) areas[c] = m.area[c];
    if (centroids2) { centroids2[2 * c] = m.cx[c]; centroids2[2 * c + 1] = m.cy[c]; }
  }
  return HG_OK;
}

int hg_mesh_order(const hg_mesh* mesh, int32_t order, int32_t* perm) {
  if (!mesh || !perm) return fail(nullptr, HG_ERR_ARG, "hg_mesh_order: null argument");
  std::vector<int> p = order_cells(mesh->m, order);
  std::memcpy(perm, p.data(), p.size() * sizeof(int32_t));
  return HG_OK;
}

namespace {
// Checks shared by hg_create and hg_ensemble_create.
int check_create_args(const hg_consts* consts, int32_t precision, int32_t device, const char* who) {
  if (precision != HG_FP64 && precision != HG_FP32C) return fail(nullptr, HG_ERR_ARG, std::string(who) + ": bad precision");
  if (consts->riemann == HG_HLLC)
    return fail(nullptr, HG_ERR_UNSUPPORTED,
                std::string(who) + ": HLLC solver not implemented (as in semi_discretize_swe_2D.jl:358-359)");
  if (consts->riemann != HG_ROE && consts->riemann != HG_HLL)
    return fail(nullptr, HG_ERR_ARG, std::string(who) + ": bad Riemann solver");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return fail(nullptr, HG_ERR_NO_DEVICE, std::string(who) + ": no CUDA device (this library has no CPU fallback)");
  if (device < 0 || device >= ndev) return fail(nullptr, HG_ERR_ARG, std::string(who) + ": bad device index");
  return HG_OK;
}

// Device set-up of a context whose host mesh is built.
int finish_create(std::unique_ptr<hg_ctx>& c, const hg_consts* consts, int32_t precision, int32_t device,
                  hg_ctx** out) {
  c->k = *consts;
  c->precision = precision;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return fail(nullptr, HG_ERR_CUDA, "hg_create: cudaSetDevice failed");
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(nullptr, HG_ERR_CUDA, "hg_create: cudaStreamCreate failed");
  int rc = ctx_setup_device(c.get());
  if (rc != HG_OK) {
    std::string msg = c->err;
    return fail(nullptr, rc, msg);
  }
  *out = c.release();
  return HG_OK;
}
}  // namespace

int hg_create(const hg_mesh_desc* desc, const hg_consts* consts, int32_t precision, int32_t device, hg_ctx** out) {
  if (!desc || !consts || !out) return fail(nullptr, HG_ERR_ARG, "hg_create: null argument");
  *out = nullptr;
  int rc = check_create_args(consts, precision, device, "hg_create");
  if (rc) return rc;
  std::unique_ptr<hg_ctx> c(new (std::nothrow) hg_ctx());
  if (!c) return fail(nullptr, HG_ERR_ARG, "hg_create: out of host memory");
  std::string err;
  rc = build_host_mesh(*desc, c->hm, err);
  if (rc != HG_OK) return fail(nullptr, rc, err);
  return finish_create(c, consts, precision, device, out);
}

int hg_ensemble_create(const hg_ensemble_desc* e, const hg_consts* consts, int32_t precision, int32_t device,
                       hg_ctx** out) {
  if (!e || !consts || !out || !e->meshes || !e->member_mesh || e->n_meshes <= 0 || e->n_members <= 0)
    return fail(nullptr, HG_ERR_ARG, "hg_ensemble_create: bad argument");
  *out = nullptr;
  for (int i = 0; i < e->n_members; ++i)
    if (e->member_mesh[i] < 0 || e->member_mesh[i] >= e->n_meshes)
      return fail(nullptr, HG_ERR_ARG, "hg_ensemble_create: member_mesh out of range");
  int rc = check_create_args(consts, precision, device, "hg_ensemble_create");
  if (rc) return rc;
  std::vector<HostMesh> meshes(e->n_meshes);
  for (int i = 0; i < e->n_meshes; ++i) {
    std::string err;
    rc = build_host_mesh(e->meshes[i], meshes[i], err);
    if (rc != HG_OK) return fail(nullptr, rc, "hg_ensemble_create: mesh " + std::to_string(i) + ": " + err);
  }
  int64_t cells = 0;
  for (int i = 0; i < e->n_members; ++i) cells += meshes[e->member_mesh[i]].nCells;
  if (cells >= (int64_t)1 << 30) return fail(nullptr, HG_ERR_ARG, "hg_ensemble_create: more than 2^30 cells");
  std::unique_ptr<hg_ctx> c(new (std::nothrow) hg_ctx());
  if (!c) return fail(nullptr, HG_ERR_ARG, "hg_ensemble_create: out of host memory");
  std::vector<const HostMesh*> parts;
  c->memberCellOff.assign(1, 0);
  c->memberInletOff.assign(1, 0);
  c->memberExitOff.assign(1, 0);
  for (int i = 0; i < e->n_members; ++i) {
    const HostMesh& m = meshes[e->member_mesh[i]];
    parts.push_back(&m);
    c->memberCellOff.push_back(c->memberCellOff.back() + m.nCells);
    c->memberInletOff.push_back(c->memberInletOff.back() + (int32_t)m.inletGroups.size());
    c->memberExitOff.push_back(c->memberExitOff.back() + (int32_t)m.exitGroups.size());
  }
  concat_host_meshes(parts, c->hm);
  return finish_create(c, consts, precision, device, out);
}

int hg_ensemble_steps(hg_ctx* ctx, int32_t nsteps, double* dts, double* t_elapsed) {
  if (!ctx || nsteps < 0) return fail(ctx, HG_ERR_ARG, "hg_ensemble_steps: bad argument");
  if (ctx->ds.nMembers == 0) return fail(ctx, HG_ERR_ARG, "hg_ensemble_steps: not an ensemble context");
  if (nsteps > ctx->ds.dtCap) return fail(ctx, HG_ERR_ARG, "hg_ensemble_steps: more steps than recorded");
  cudaSetDevice(ctx->device);
  const size_t M = (size_t)ctx->ds.nMembers;
  if (dts && nsteps > 0)
    HG_CUDA(ctx, cudaMemcpyAsync(dts, ctx->ds.dtHistM, (size_t)nsteps * M * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  if (t_elapsed) HG_CUDA(ctx, cudaMemcpyAsync(t_elapsed, ctx->ds.tM, M * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return HG_OK;
}

int hg_ensemble_layout(const hg_ctx* ctx, int32_t* n_members, int32_t* cell_offset, int32_t* inlet_offset,
                       int32_t* exit_offset) {
  if (!ctx || !n_members) return fail(nullptr, HG_ERR_ARG, "hg_ensemble_layout: null argument");
  const bool ens = !ctx->memberCellOff.empty();
  const int M = ens ? (int)ctx->memberCellOff.size() - 1 : 1;
  *n_members = M;
  for (int i = 0; i <= M; ++i) {
    if (cell_offset) cell_offset[i] = ens ? ctx->memberCellOff[i] : (i ? ctx->n : 0);
    if (inlet_offset) inlet_offset[i] = ens ? ctx->memberInletOff[i] : (i ? ctx->dm.nInlet : 0);
    if (exit_offset) exit_offset[i] = ens ? ctx->memberExitOff[i] : (i ? ctx->dm.nExit : 0);
  }
  return HG_OK;
}

int hg_destroy(hg_ctx* ctx) {
  if (ctx) cudaSetDevice(ctx->device);
  delete ctx;
  return HG_OK;
}

int hg_sizes(const hg_ctx* ctx, int32_t* sizes8) {
  if (!ctx || !sizes8) return fail(nullptr, HG_ERR_ARG, "hg_sizes: null argument");
  return sizes_of(ctx->hm, sizes8);
}

int hg_set_still_water(hg_ctx* ctx, const double* wstill) {
  if (!ctx || !wstill) return fail(ctx, HG_ERR_ARG, "hg_set_still_water: null argument");
  cudaSetDevice(ctx->device);
  for (int i = 0; i < ctx->n; ++i) ctx->hstill[i] = wstill[i] - ctx->zbCell[i];   // process_ICs_2D.jl:55
  return upload_cells(ctx);
}

int hg_set_manning_zones(hg_ctx* ctx, const int32_t* mat_id, int32_t n_zones, const double* n_zone) {
  if (!ctx || !mat_id || !n_zone || n_zones <= 0) return fail(ctx, HG_ERR_ARG, "hg_set_manning_zones: bad argument");
  for (int i = 0; i < ctx->n; ++i) {
    if (mat_id[i] < 0 || mat_id[i] >= n_zones)
      return fail(ctx, HG_ERR_ARG, "hg_set_manning_zones: cell " + std::to_string(i) + " has zone " +
                                       std::to_string(mat_id[i]) + " outside [0, n_zones)");
  }
  cudaSetDevice(ctx->device);
  for (int i = 0; i < ctx->n; ++i) ctx->manning[i] = n_zone[mat_id[i]];   // process_ManningN_2D.jl:259
  return upload_cells(ctx);
}

int hg_set_manning_cells(hg_ctx* ctx, const double* n) {
  if (!ctx || !n) return fail(ctx, HG_ERR_ARG, "hg_set_manning_cells: null argument");
  cudaSetDevice(ctx->device);
  ctx->manning.assign(n, n + ctx->n);
  return upload_cells(ctx);
}

int hg_set_zb_cells(hg_ctx* ctx, const double* zb) {
  if (!ctx || !zb) return fail(ctx, HG_ERR_ARG, "hg_set_zb_cells: null argument");
  cudaSetDevice(ctx->device);
  ctx->zbCell.assign(zb, zb + ctx->n);
  compute_bed(ctx->hm, ctx->zbCell, ctx->s0x, ctx->s0y);
  return upload_cells(ctx);
}

int hg_set_inlet_q(hg_ctx* ctx, const double* q, int32_t n) {
  if (!ctx || (n > 0 && !q) || n != (int32_t)ctx->inletQ.size())
    return fail(ctx, HG_ERR_ARG, "hg_set_inlet_q: expected one value per inlet-Q boundary");
  cudaSetDevice(ctx->device);
  ctx->inletQ.assign(q, q + n);
  return upload_boundary_values(ctx);
}

int hg_set_exit_wse(hg_ctx* ctx, const double* w, int32_t n) {
  if (!ctx || (n > 0 && !w) || n != (int32_t)ctx->exitWse.size())
    return fail(ctx, HG_ERR_ARG, "hg_set_exit_wse: expected one value per exit-H boundary");
  cudaSetDevice(ctx->device);
  ctx->exitWse.assign(w, w + n);
  return upload_boundary_values(ctx);
}

int hg_resistance_grad(const hg_ctx* ctx, double* g_params) {
  if (!ctx || !g_params) return fail(nullptr, HG_ERR_ARG, "hg_resistance_grad: null argument");
  for (int k = 0; k < 4; ++k) g_params[k] = ctx->resGrad[k];
  return HG_OK;
}

int hg_ude_grad(const hg_ctx* ctx, double* g_params, int64_t n_params) {
  if (!ctx || (!g_params && n_params > 0)) return fail(nullptr, HG_ERR_ARG, "hg_ude_grad: null argument");
  if (n_params != (int64_t)ctx->udeParams)
    return fail(nullptr, HG_ERR_ARG, "hg_ude_grad: the closure has " + std::to_string(ctx->udeParams) + " parameters");
  for (int64_t k = 0; k < n_params; ++k) g_params[k] = k < (int64_t)ctx->udeGrad.size() ? ctx->udeGrad[k] : 0.0;
  return HG_OK;
}

int hg_set_dt_min(hg_ctx* ctx, double dt_min) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_dt_min: null context");
  if (!(dt_min >= 0.0) || !std::isfinite(dt_min)) return fail(ctx, HG_ERR_ARG, "hg_set_dt_min: dt_min must be >= 0");
  ctx->ds.dtMin = dt_min;
  ctx->graphValid = false;   // captured launches hold the scalars descriptor by value
  return HG_OK;
}

int hg_set_riemann_solver(hg_ctx* ctx, int32_t solver) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_riemann_solver: null context");
  if (solver == HG_HLLC)
    return fail(ctx, HG_ERR_UNSUPPORTED,
                "hg_set_riemann_solver: HLLC solver not implemented (as in semi_discretize_swe_2D.jl:358-359)");
  if (solver != HG_ROE && solver != HG_HLL) return fail(ctx, HG_ERR_ARG, "hg_set_riemann_solver: expected HG_ROE or HG_HLL");
  ctx->k.riemann = solver;
  ctx->dm.riemann = solver;
  ctx->graphValid = false;   // captured launches hold the mesh descriptor by value
  return HG_OK;
}

int hg_set_inlet_hydrograph(hg_ctx* ctx, int32_t group, int32_t n, const double* t, const double* q) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_inlet_hydrograph: null context");
  const int ng = ctx->dm.nInlet;
  if (group < 0 || group >= ng || n < 0 || (n > 0 && (!t || !q)))
    return fail(ctx, HG_ERR_ARG, "hg_set_inlet_hydrograph: bad group or points");
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(t[i]) || !std::isfinite(q[i]) || (i > 0 && !(t[i] > t[i - 1])))
      return fail(ctx, HG_ERR_ARG, "hg_set_inlet_hydrograph: times must increase, values be finite");
  cudaSetDevice(ctx->device);
  ctx->hydro.resize(ng);
  ctx->hydro[group].assign(t, t + n);
  ctx->hydro[group].insert(ctx->hydro[group].end(), q, q + n);
  std::vector<int32_t> off(ng + 1, 0);
  std::vector<double> tt, qq;
  for (int g = 0; g < ng; ++g) {
    const std::vector<double>& h = ctx->hydro[g];
    const size_t k = h.size() / 2;
    tt.insert(tt.end(), h.begin(), h.begin() + k);
    qq.insert(qq.end(), h.begin() + k, h.end());
    off[g + 1] = (int32_t)tt.size();
  }
  ctx->dm.nHydro = (int32_t)tt.size();
  if (!tt.empty()) {
    if (tt.size() > ctx->hydroCap) {
      HG_CUDA(ctx, dalloc(ctx, &ctx->d_hydroT, tt.size()));
      HG_CUDA(ctx, dalloc(ctx, &ctx->d_hydroQ, tt.size()));
      ctx->hydroCap = tt.size();
    }
    if (!ctx->d_hydroOff) HG_CUDA(ctx, dalloc(ctx, &ctx->d_hydroOff, (size_t)ng + 1));
    HG_CUDA(ctx, upload(ctx, ctx->d_hydroOff, off));
    HG_CUDA(ctx, upload(ctx, ctx->d_hydroT, tt));
    HG_CUDA(ctx, upload(ctx, ctx->d_hydroQ, qq));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->dm.hydroOff = ctx->d_hydroOff;
    ctx->dm.hydroT = ctx->d_hydroT;
    ctx->dm.hydroQ = ctx->d_hydroQ;
  }
  ctx->graphValid = false;
  return upload_boundary_values(ctx);   // groups without a hydrograph: back to their constant discharge
}

int hg_set_manning_function(hg_ctx* ctx, int32_t kind, const double* params, int32_t n_params, const double* ks) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_manning_function: null context");
  cudaSetDevice(ctx->device);
  if (kind == HG_RES_CONSTANT) {   // back to the cells' n
    ctx->dm.res = ResDev{};
    ctx->graphValid = false;
    return upload_cells(ctx);
  }
  if (kind < HG_RES_POWER_LAW || kind > HG_RES_H_UMAG_KS)
    return fail(ctx, HG_ERR_ARG, "hg_set_manning_function: kind must be one of HG_RES_CONSTANT..HG_RES_H_UMAG_KS");
  ResDev r;
  r.kind = kind;
  if (kind == HG_RES_H_UMAG_KS) {
    if (!ks || !all_positive(ks, ctx->n))
      return fail(ctx, HG_ERR_ARG, "hg_set_manning_function: h_Umag_ks needs a positive ks per cell");
  } else {
    const int need = kind == HG_RES_SIGMOID ? 4 : 3;
    if (!params || n_params < need)
      return fail(ctx, HG_ERR_ARG, "hg_set_manning_function: params = {n_lower, n_upper, k[, h_mid]}");
    // the reference's own checks (process_ManningN_2D.jl:150,165,181-182)
    if (!(params[2] > 0.0)) return fail(ctx, HG_ERR_ARG, "k must be a positive scaling factor");
    if (kind == HG_RES_SIGMOID && !(params[3] > 0.0)) return fail(ctx, HG_ERR_ARG, "h_mid must be a positive water depth");
    for (int i = 0; i < need; ++i) r.p[i] = params[i];
  }
  return install_resistance(ctx, r, kind == HG_RES_H_UMAG_KS ? ks : nullptr, nullptr, 0);
}

int hg_set_ude(hg_ctx* ctx, const hg_ude_desc* u) {
  if (!ctx || !u) return fail(ctx, HG_ERR_ARG, "hg_set_ude: null argument");
  if (u->kind < HG_RES_UDE_MANNING_H || u->kind > HG_RES_UDE_FLOW_RESISTANCE)
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: kind must be one of the HG_RES_UDE_* values");
  if (u->n_hidden < 0 || u->n_hidden > kResMaxLayers || (u->n_hidden > 0 && (!u->hidden || !u->activation)))
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: 0 to 4 hidden layers");
  ResDev r;
  r.kind = u->kind;
  r.inDim = u->kind == HG_RES_UDE_MANNING_H ? 1 : u->kind == HG_RES_UDE_MANNING_H_UMAG_KS ? 3 : 2;
  r.nHidden = u->n_hidden;
  r.overBatch = u->layernorm_over_batch ? 1 : 0;
  r.lnEps = (double)1e-5f;   // Lux's LayerNorm default epsilon (Float32)
  int din = r.inDim, count = 0;
  for (int l = 0; l < u->n_hidden; ++l) {
    const int w = u->hidden[l];
    if (w < 1 || w > kResMaxWidth) return fail(ctx, HG_ERR_ARG, "hg_set_ude: hidden widths must be 1..16");
    if (u->activation[l] < HG_ACT_RELU || u->activation[l] > HG_ACT_SOFTPLUS)
      return fail(ctx, HG_ERR_ARG, "hg_set_ude: unknown activation");
    r.width[l] = w;
    r.act[l] = u->activation[l];
    count += w * din + 3 * w;
    din = w;
  }
  count += din + 1;
  if (!u->params || u->n_params != count)
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: expected " + std::to_string(count) + " network parameters");
  const double* b[3] = {u->h_bounds, u->u_bounds, u->ks_bounds};
  for (int i = 0; i < 3; ++i) {
    r.lo[i] = b[i][0];
    r.hi[i] = b[i][1];
  }
  if (!(r.hi[0] != r.lo[0]) || (r.inDim > 1 && !(r.hi[1] != r.lo[1])) ||
      (u->kind == HG_RES_UDE_MANNING_H_UMAG_KS && !(r.hi[2] != r.lo[2])))
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: empty input bounds");
  if (u->kind == HG_RES_UDE_FLOW_RESISTANCE && !(r.hi[0] * r.hi[1] != r.lo[0] * r.lo[1]))
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: empty discharge bounds");
  if (u->kind == HG_RES_UDE_MANNING_H_UMAG_KS && !u->ks_cells)
    return fail(ctx, HG_ERR_ARG, "hg_set_ude: ManningN_h_Umag_ks needs ks per cell");
  r.outLo = u->output_bounds[0];
  r.outHi = u->output_bounds[1];
  cudaSetDevice(ctx->device);
  int rc = install_resistance(ctx, r, u->kind == HG_RES_UDE_MANNING_H_UMAG_KS ? u->ks_cells : nullptr, u->params,
                              u->n_params);
  if (rc) return rc;
  // n returns to the cells' values where the closure replaces only the friction
  return u->kind == HG_RES_UDE_FLOW_RESISTANCE ? upload_cells(ctx) : HG_OK;
}

int hg_final_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                           const hg_final_obs* obs, double* parts, double* g_manning_cells, double* g_zb,
                           double* g_inletq, double* Q_final) {
  if (!ctx || !Q0 || nsteps <= 0 || !(dt > 0) || !obs || !parts || (!obs->wse && !(obs->u && obs->v)) ||
      (!obs->u != !obs->v))
    return fail(ctx, HG_ERR_ARG, "hg_final_loss_and_grad: bad argument");
  cudaSetDevice(ctx->device);
  FinalObs fo;
  fo.wse = obs->wse;
  fo.u = obs->u;
  fo.v = obs->v;
  fo.zbw = obs->zb_wse;
  double loss = 0.0;
  return adjoint_loss_and_grad(ctx, Q0, nsteps, dt, ckpt_every, nullptr, nullptr, 0, &loss, g_manning_cells, g_zb,
                               g_inletq, Q_final, &fo, parts);
}

int hg_final_vjp(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every, const double* lambda,
                 double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final) {
  if (!ctx || !Q0 || nsteps <= 0 || !(dt > 0) || !lambda) return fail(ctx, HG_ERR_ARG, "hg_final_vjp: bad argument");
  cudaSetDevice(ctx->device);
  FinalObs fo;
  fo.lam = lambda;
  double loss = 0.0, parts[3];
  return adjoint_loss_and_grad(ctx, Q0, nsteps, dt, ckpt_every, nullptr, nullptr, 0, &loss, g_manning_cells, g_zb,
                               g_inletq, Q_final, &fo, parts);
}

int hg_get_bed(hg_ctx* ctx, double* zb, double* S0, double* man, double* hstill) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_get_bed: null context");
  for (int i = 0; i < ctx->n; ++i) {
    if (zb) zb[i] = ctx->zbCell[i];
    if (S0) { S0[2 * i] = ctx->s0x[i]; S0[2 * i + 1] = ctx->s0y[i]; }
    if (man) man[i] = ctx->manning[i];
    if (hstill) hstill[i] = ctx->hstill[i];
  }
  return HG_OK;
}

int hg_check_initial_state(hg_ctx* ctx, const double* Q) {
  if (!ctx || !Q) return fail(ctx, HG_ERR_ARG, "hg_check_initial_state: null argument");
  for (int i = 0; i < ctx->n; ++i) {
    const double h = Q[i] + ctx->hstill[i];
    if (!std::isfinite(Q[i]) || !std::isfinite(Q[ctx->n + i]) || !std::isfinite(Q[2 * ctx->n + i]))
      return fail(ctx, HG_ERR_STATE, "initial state is not finite at cell " + std::to_string(i));
    if (h < ctx->k.h_small)
      return fail(ctx, HG_ERR_STATE, "initial depth " + std::to_string(h) + " at cell " + std::to_string(i) +
                                         " is below h_small (process_ICs_2D.jl:97-99)");
  }
  return HG_OK;
}

int hg_rhs(hg_ctx* ctx, const double* Q, double t, double* dQ) {
  if (!ctx || !Q || !dQ) return fail(ctx, HG_ERR_ARG, "hg_rhs: null argument");
  cudaSetDevice(ctx->device);
  launch_reset_scalars(ctx->ds, ctx->stream);
  ctx->launches += launch_hydrograph(ctx->dm, ctx->ds, kHydroAt, t, ctx->stream);
  int rc = enqueue_upload(ctx, Q);
  if (rc) return rc;
  if (ctx->precision == HG_FP64) {
    launch_inlet_total_f64(ctx->dm, ctx->ds, ctx->QA, ctx->stream);
    launch_stage_f64(ctx->dm, ctx->ds, kModeRhs, ctx->QA, nullptr, ctx->QB, false, ctx->stream);
    launch_scatter_state_f64(ctx->n, ctx->d_perm, ctx->QB, ctx->Quser, ctx->stream);
  } else {
    launch_inlet_total_f32(ctx->dm, ctx->ds, xa(ctx), ctx->stream);
    launch_stage_f32(ctx->dm, ctx->ds, kModeRhs, xa(ctx), StateF32{}, StateF32{}, ctx->QB, false, ctx->stream);
    launch_scatter_state_f64(ctx->n, ctx->d_perm, ctx->QB, ctx->Quser, ctx->stream);
  }
  ctx->launches += 3 + rhs_prep_launches(ctx);   // reset, stage, scatter; resistance, inlet totals
  HG_CUDA(ctx, cudaMemcpyAsync(dQ, ctx->Quser, (size_t)3 * ctx->n * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  HG_CUDA(ctx, cudaGetLastError());
  return check_flags(ctx);
}

int hg_integrate(hg_ctx* ctx, double* Q, double /*t0*/, int32_t nsteps, int32_t method, double dt, double cfl,
                 int32_t save_every, double* saves, double* dts_out) {
  if (!ctx || !Q || nsteps < 0) return fail(ctx, HG_ERR_ARG, "hg_integrate: bad argument");
  if (method != 0 && method != 1) return fail(ctx, HG_ERR_ARG, "hg_integrate: method must be 0 (SSP-RK2) or 1 (Euler)");
  if (save_every > 0 && !saves) return fail(ctx, HG_ERR_ARG, "hg_integrate: saves is NULL");
  if (dt <= 0 && !(cfl > 0)) return fail(ctx, HG_ERR_ARG, "hg_integrate: need dt > 0 or cfl > 0");
  cudaSetDevice(ctx->device);
  int rc = ensure_dt_capacity(ctx, nsteps);
  if (rc) return rc;
  launch_reset_scalars(ctx->ds, ctx->stream);
  rc = enqueue_upload(ctx, Q);
  if (rc) return rc;
  const bool cflMode = dt <= 0;
  ctx->cflPrimed = false;
  rc = begin_steps(ctx, method == 0, dt, cfl);
  if (rc) return rc;
  int saved = 0;
  for (int s = 0; s < nsteps; ++s) {
    if (method == 0) enqueue_rk2_step(ctx, cflMode, cfl);
    else enqueue_euler_step(ctx, cflMode, cfl);
    if (save_every > 0 && (s + 1) % save_every == 0) {
      rc = enqueue_download(ctx, saves + (size_t)saved * 3 * ctx->n);
      if (rc) return rc;
      ++saved;
    }
  }
  ctx->cflPrimed = cflMode;
  rc = enqueue_download(ctx, Q);
  if (rc) return rc;
  if (dts_out && nsteps > 0)
    HG_CUDA(ctx, cudaMemcpyAsync(dts_out, ctx->ds.dtHist, (size_t)nsteps * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  HG_CUDA(ctx, cudaGetLastError());
  return check_flags(ctx);
}

int hg_state_upload(hg_ctx* ctx, const double* Q) {
  if (!ctx || !Q) return fail(ctx, HG_ERR_ARG, "hg_state_upload: null argument");
  cudaSetDevice(ctx->device);
  launch_reset_scalars(ctx->ds, ctx->stream);
  int rc = enqueue_upload(ctx, Q);
  if (rc) return rc;
  ctx->cflPrimed = false;
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return HG_OK;
}

int hg_state_download(hg_ctx* ctx, double* Q) {
  if (!ctx || !Q) return fail(ctx, HG_ERR_ARG, "hg_state_download: null argument");
  cudaSetDevice(ctx->device);
  int rc = enqueue_download(ctx, Q);
  if (rc) return rc;
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_flags(ctx);
}

int hg_advance(hg_ctx* ctx, int32_t nsteps, double dt, double cfl, int32_t graph) {
  if (!ctx || nsteps < 0) return fail(ctx, HG_ERR_ARG, "hg_advance: bad argument");
  if (dt <= 0 && !(cfl > 0)) return fail(ctx, HG_ERR_ARG, "hg_advance: need dt > 0 or cfl > 0");
  cudaSetDevice(ctx->device);
  const bool cflMode = dt <= 0;
  int rc0 = begin_steps(ctx, true, dt, cfl);
  if (rc0) return rc0;
  int done = 0;
  if (graph) {
    const int K = kGraphSteps;
    if (fused(ctx) && ctx->graphValid && ctx->parity != ctx->graphParity && nsteps > K) {
      enqueue_rk2_step(ctx, cflMode, cfl);   // bring the CFL-buffer parity to the graph's
      ++done;
    }
    if (nsteps - done >= K) {
      if (!ctx->graphValid || ctx->graphCflMode != cflMode || ctx->graphCfl != cfl ||
          (fused(ctx) && ctx->parity != ctx->graphParity)) {
        if (ctx->graphExec) {
          cudaGraphExecDestroy(ctx->graphExec);
          ctx->graphExec = nullptr;
        }
        cudaGraph_t g;
        ctx->graphParity = ctx->parity;
        HG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int64_t before = ctx->launches;
        for (int s = 0; s < K; ++s) enqueue_rk2_step(ctx, cflMode, cfl);
        ctx->graphLaunches = ctx->launches - before;
        ctx->launches = before;
        HG_CUDA(ctx, cudaStreamEndCapture(ctx->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&ctx->graphExec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(ctx, HG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        ctx->graphValid = true;
        ctx->graphCflMode = cflMode;
        ctx->graphCfl = cfl;
      }
      for (; done + K <= nsteps; done += K) {
        HG_CUDA(ctx, cudaGraphLaunch(ctx->graphExec, ctx->stream));
        ctx->launches += ctx->graphLaunches;
      }
      ctx->parity = ctx->graphParity;   // K is even: a graph ends on the parity it starts with
    }
  }
  for (; done < nsteps; ++done) enqueue_rk2_step(ctx, cflMode, cfl);
  ctx->cflPrimed = cflMode;
  HG_CUDA(ctx, cudaGetLastError());
  return HG_OK;
}

int hg_synchronize(hg_ctx* ctx) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_synchronize: null context");
  cudaSetDevice(ctx->device);
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_flags(ctx);
}

int hg_elapsed_time(hg_ctx* ctx, double* t) {
  if (!ctx || !t) return fail(ctx, HG_ERR_ARG, "hg_elapsed_time: null argument");
  cudaSetDevice(ctx->device);
  HG_CUDA(ctx, cudaMemcpyAsync(t, ctx->ds.tSum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return HG_OK;
}

int hg_launch_count(const hg_ctx* ctx, int64_t* count) {
  if (!ctx || !count) return fail(nullptr, HG_ERR_ARG, "hg_launch_count: null argument");
  *count = ctx->launches;
  return HG_OK;
}

int hg_flush_l2(hg_ctx* ctx) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_flush_l2: null context");
  cudaSetDevice(ctx->device);
  ctx->launches += launch_flush(ctx->flushBuf, ctx->flushBytes, ctx->stream);
  HG_CUDA(ctx, cudaGetLastError());
  return HG_OK;
}

int hg_advance_timed(hg_ctx* ctx, int32_t nsteps, double dt, double cfl, int32_t flush_l2, double* total_ms) {
  if (!ctx || nsteps <= 0 || !total_ms) return fail(ctx, HG_ERR_ARG, "hg_advance_timed: bad argument");
  if (dt <= 0 && !(cfl > 0)) return fail(ctx, HG_ERR_ARG, "hg_advance_timed: need dt > 0 or cfl > 0");
  cudaSetDevice(ctx->device);
  const bool cflMode = dt <= 0;
  int rc0 = begin_steps(ctx, true, dt, cfl);
  if (rc0) return rc0;
  std::vector<cudaEvent_t> ev(2 * (size_t)nsteps, nullptr);
  for (auto& e : ev) HG_CUDA(ctx, cudaEventCreate(&e));
  for (int s = 0; s < nsteps; ++s) {
    if (flush_l2) ctx->launches += launch_flush(ctx->flushBuf, ctx->flushBytes, ctx->stream);
    cudaEventRecord(ev[2 * s], ctx->stream);
    enqueue_rk2_step(ctx, cflMode, cfl);
    cudaEventRecord(ev[2 * s + 1], ctx->stream);
  }
  ctx->cflPrimed = cflMode;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  double total = 0.0;
  for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]);
    total += ms;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return fail(ctx, HG_ERR_CUDA, std::string("hg_advance_timed: ") + cudaGetErrorString(e));
  *total_ms = total;
  return check_flags(ctx);
}

int hg_autotune(hg_ctx* ctx, int32_t reps, int32_t* kernel) {
  if (!ctx || reps < 0) return fail(ctx, HG_ERR_ARG, "hg_autotune: bad argument");
  cudaSetDevice(ctx->device);
  if (reps > 0) {
    int rc = autotune_stage(ctx, reps, false);
    if (rc) return rc;
  }
  if (kernel) *kernel = stage_kernel_forced() >= 0 ? stage_kernel_forced() : ctx->dm.stageKernel;
  return HG_OK;
}

int hg_autotune_info(const hg_ctx* ctx, int32_t* kernel, int32_t* variant, int32_t* source) {
  if (!ctx) return fail(nullptr, HG_ERR_ARG, "hg_autotune_info: null context");
  const bool forced = stage_kernel_forced() >= 0 || stage_variant_forced() >= 0;
  if (kernel) *kernel = stage_kernel_forced() >= 0 ? stage_kernel_forced() : ctx->dm.stageKernel;
  if (variant) *variant = stage_variant_forced() >= 0 ? stage_variant_forced() : ctx->dm.stageVariant;
  if (source) *source = forced ? 3 : ctx->tuneSource;
  return HG_OK;
}

int hg_set_stage_family(hg_ctx* ctx, int32_t family) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_stage_family: null context");
  if (family != 0 && family != 1) return fail(ctx, HG_ERR_ARG, "hg_set_stage_family: 0 (gather) or 1 (face)");
  if (family == 1 && !ctx->dm.FL) return fail(ctx, HG_ERR_UNSUPPORTED, "hg_set_stage_family: no face tables for this mesh");
  ctx->stageFamily = family;
  set_stage_choice(ctx, family == 1 ? TuneChoice{kStageFace, 0}
                                    : TuneChoice{ctx->dm.SLp ? kStagePipe : kStageGather, 0});
  ctx->stageTuned = false;   // the next RK2 steps tune (or read the cache) within the family
  ctx->tuneSource = 0;
  return HG_OK;
}

int hg_time_stage_kernel(hg_ctx* ctx, int32_t n, int32_t flush_l2, double* avg_ms) {
  if (!ctx || n <= 0 || !avg_ms) return fail(ctx, HG_ERR_ARG, "hg_time_stage_kernel: bad argument");
  cudaSetDevice(ctx->device);
  cudaEvent_t a, b;
  HG_CUDA(ctx, cudaEventCreate(&a));
  HG_CUDA(ctx, cudaEventCreate(&b));
  double total = 0.0;
  if (fused(ctx)) {   // conveyance totals of the resident state
    DevMesh m = ctx->dm;
    m.totalA = ctx->d_tot;
    launch_inlet_total_f32(m, ctx->ds, xa(ctx), ctx->stream);
    ctx->launches += ctx->dm.nInlet > 0 ? 1 : 0;
  }
  for (int i = 0; i < n; ++i) {
    if (flush_l2) ctx->launches += launch_flush(ctx->flushBuf, ctx->flushBytes, ctx->stream);
    cudaEventRecord(a, ctx->stream);
    if (ctx->precision == HG_FP64) {
      launch_stage_f64(ctx->dm, ctx->ds, kModeStage1, ctx->QA, nullptr, ctx->QB, false, ctx->stream);
    } else if (fused(ctx)) {
      // the stage-1 launch of a fused step at the current dt, without the step bookkeeping
      StageFuse f;
      f.partials = ctx->d_partials;
      f.ticket = ctx->d_ticket;
      f.blockSlot = ctx->d_blockSlot;
      f.nSlots = ctx->nSlots;
      f.nWarps = ctx->nWarps;
      f.totalIn = ctx->d_tot;
      f.totalOut = ctx->d_tot + kMaxFusedInlets;
      launch_stage_f32_fused(ctx->dm, ctx->ds, kModeStage1, xa(ctx), StateF32{}, xb(ctx), f, ctx->stream);
    } else {
      launch_stage_f32(ctx->dm, ctx->ds, kModeStage1, xa(ctx), StateF32{}, xb(ctx), nullptr, false, ctx->stream);
    }
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    total += ms;
    ctx->launches += 1;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *avg_ms = total / n;
  HG_CUDA(ctx, cudaGetLastError());
  return HG_OK;
}

int hg_time_vjp_kernel(hg_ctx* ctx, int32_t n, int32_t flush_l2, double* avg_ms) {
  if (!ctx || n <= 0 || !avg_ms) return fail(ctx, HG_ERR_ARG, "hg_time_vjp_kernel: bad argument");
  cudaSetDevice(ctx->device);
  return adjoint_time_vjp(ctx, n, flush_l2, avg_ms);
}

int hg_set_adjoint_tape(hg_ctx* ctx, int64_t bytes) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_tape: null context");
  cudaSetDevice(ctx->device);
  ctx->adjTapeBytes = bytes < 0 ? -1 : bytes;
  adjoint_release_tape(ctx);
  return HG_OK;
}

int hg_set_adjoint_integrator(hg_ctx* ctx, int32_t integrator) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_integrator: null context");
  if (integrator != HG_ADJ_SSPRK2 && integrator != HG_ADJ_TSIT5)
    return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_integrator: HG_ADJ_SSPRK2 or HG_ADJ_TSIT5");
  ctx->adjIntegrator = integrator;
  return HG_OK;
}

int hg_set_adjoint_steps(hg_ctx* ctx, const double* dts, int32_t n) {
  if (!ctx) return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_steps: null context");
  if (n < 0 || (n > 0 && !dts)) return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_steps: bad argument");
  for (int i = 0; i < n; ++i)
    if (!(dts[i] > 0) || !std::isfinite(dts[i]))
      return fail(ctx, HG_ERR_ARG, "hg_set_adjoint_steps: step sizes must be positive and finite");
  ctx->adjSteps.assign(dts, dts + n);
  return HG_OK;
}

int hg_tsit5_steps(const hg_ctx* ctx, double* dts, int32_t cap, int32_t* count) {
  if (!ctx || cap < 0 || (cap > 0 && !dts)) return HG_ERR_ARG;
  const size_t m = std::min(ctx->tsit5Steps.size(), (size_t)cap);
  for (size_t i = 0; i < m; ++i) dts[i] = ctx->tsit5Steps[i];
  if (count) *count = (int32_t)ctx->tsit5Steps.size();
  return HG_OK;
}

int hg_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                     const int32_t* probe_cells, const double* obs, int32_t n_probe, double* loss,
                     double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final) {
  if (!ctx || !Q0 || nsteps <= 0 || !(dt > 0) || n_probe < 0 || (n_probe > 0 && (!probe_cells || !obs)) || !loss)
    return fail(ctx, HG_ERR_ARG, "hg_loss_and_grad: bad argument");
  for (int i = 0; i < n_probe; ++i)
    if (probe_cells[i] < 0 || probe_cells[i] >= ctx->n) return fail(ctx, HG_ERR_ARG, "hg_loss_and_grad: bad probe id");
  cudaSetDevice(ctx->device);
  return adjoint_loss_and_grad(ctx, Q0, nsteps, dt, ckpt_every, probe_cells, obs, n_probe, loss, g_manning_cells, g_zb,
                               g_inletq, Q_final);
}

int hg_pinned_alloc(int64_t bytes, void** out) {
  if (!out || bytes <= 0) return fail(nullptr, HG_ERR_ARG, "hg_pinned_alloc: bad argument");
  if (cudaMallocHost(out, (size_t)bytes) != cudaSuccess) return fail(nullptr, HG_ERR_CUDA, "cudaMallocHost failed");
  return HG_OK;
}

int hg_pinned_free(void* p) {
  if (p) cudaFreeHost(p);
  return HG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Device setup (called by hg_create)
// ---------------------------------------------------------------------------
int ctx_setup_device(hg_ctx* c) {
  const HostMesh& m = c->hm;
  const int N = m.nCells;
  c->n = N;
  c->perm = c->memberCellOff.size() > 2 ? order_cells_ranges(m, c->k.order, c->memberCellOff)
                                        : order_cells(m, c->k.order);
  c->inv.assign(N, 0);
  for (int i = 0; i < N; ++i) c->inv[c->perm[i]] = i;
  // Boundary faces, numbered by face id.
  std::vector<int> bfOf(m.nFaces, -1);
  int nbf = 0;
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceC1[f] < 0) bfOf[f] = nbf++;
  std::vector<int> groupOf(m.bnd.size(), 0);
  for (size_t g = 0; g < m.inletGroups.size(); ++g) groupOf[m.inletGroups[g]] = (int)g;
  for (size_t g = 0; g < m.exitGroups.size(); ++g) groupOf[m.exitGroups[g]] = (int)g;
  std::vector<int32_t> bfInfo(nbf, 0);
  std::vector<double> bfLp23(nbf, 0.0), bfLp53(nbf, 0.0);
  for (int f = 0; f < m.nFaces; ++f) {
    if (bfOf[f] < 0) continue;
    const int bi = m.faceBnd[f];
    const int type = m.bnd[bi].bc;
    bfInfo[bfOf[f]] = type | (groupOf[bi] << 2);
    if (type == HG_BC_EXITH) {
      c->exitBf.push_back(bfOf[f]);
      c->exitCell.push_back(m.faceC0[f]);
      c->exitGrp.push_back(groupOf[bi]);
    }
    if (type == HG_BC_INLETQ) {
      bfLp23[bfOf[f]] = std::pow(m.faceLen[f], 2.0 / 3.0);
      bfLp53[bfOf[f]] = std::pow(m.faceLen[f], 5.0 / 3.0);
    }
  }
  const int S = m.maxCellFaces;
  std::vector<int32_t> nb((size_t)S * N, INT32_MIN);
  std::vector<double> snx((size_t)S * N, 0.0), sny((size_t)S * N, 0.0), slen((size_t)S * N, 0.0);
  for (int c2 = 0; c2 < N; ++c2) {
    const int o = c->perm[c2];
    for (int k = 0; k < m.ncf[o]; ++k) {
      const size_t src = (size_t)o * 8 + k, dst = (size_t)k * N + c2;
      const int f = m.cf[src];
      nb[dst] = m.nbr[src] >= 0 ? c->inv[m.nbr[src]] : -1 - bfOf[f];
      snx[dst] = m.snx[src];
      sny[dst] = m.sny[src];
      slen[dst] = m.faceLen[f];
    }
  }
  std::vector<int32_t> inletOff(1, 0), inletCell;
  std::vector<double> inletLp53;
  for (int g : m.inletGroups) {
    for (int f : m.bnd[g].faces) {
      inletCell.push_back(c->inv[m.faceC0[f]]);
      inletLp53.push_back(std::pow(m.faceLen[f], 5.0 / 3.0));
    }
    inletOff.push_back((int32_t)inletCell.size());
  }
  std::vector<double> area = to_device_order(c, m.area.data());

  // Parameters with their defaults: zb from the nodes, hstill 0 until set,
  // Manning n 0.03 until set, boundary values 0 until set.
  c->zbCell = m.zbCell;
  compute_bed(m, c->zbCell, c->s0x, c->s0y);
  c->hstill.assign(N, 0.0);
  c->manning.assign(N, 0.03);
  c->inletQ.assign(m.inletGroups.size(), 0.0);
  c->exitWse.assign(m.exitGroups.size(), 0.0);

  int32_t* d_nb; double *d_snx, *d_sny, *d_slen, *d_area, *d_lp23, *d_lp53, *d_bflp53; float* d_lp23f; float4* d_SL;
  int32_t *d_bfInfo, *d_inletOff, *d_inletCell;
  HG_CUDA(c, dalloc(c, &d_nb, nb.size()));
  HG_CUDA(c, dalloc(c, &d_snx, snx.size()));
  HG_CUDA(c, dalloc(c, &d_sny, sny.size()));
  HG_CUDA(c, dalloc(c, &d_slen, slen.size()));
  HG_CUDA(c, dalloc(c, &d_SL, nb.size()));
  HG_CUDA(c, dalloc(c, &d_area, (size_t)N));
  HG_CUDA(c, dalloc(c, &d_bfInfo, (size_t)std::max(nbf, 1)));
  HG_CUDA(c, dalloc(c, &c->d_bfExitRel, (size_t)std::max(nbf, 1)));
  c->h_bfExitRel.assign(std::max(nbf, 1), 0.0f);
  HG_CUDA(c, dalloc(c, &d_lp23, (size_t)std::max(nbf, 1)));
  HG_CUDA(c, dalloc(c, &d_lp23f, (size_t)std::max(nbf, 1)));
  HG_CUDA(c, dalloc(c, &d_bflp53, (size_t)std::max(nbf, 1)));
  HG_CUDA(c, dalloc(c, &d_inletOff, inletOff.size()));
  HG_CUDA(c, dalloc(c, &d_inletCell, std::max<size_t>(inletCell.size(), 1)));
  HG_CUDA(c, dalloc(c, &d_lp53, std::max<size_t>(inletLp53.size(), 1)));
  for (double** p : {&c->d_hst, &c->d_zb, &c->d_man, &c->d_s0x, &c->d_s0y}) HG_CUDA(c, dalloc(c, p, (size_t)N));
  HG_CUDA(c, dalloc(c, &c->d_CP, (size_t)N));
  HG_CUDA(c, dalloc(c, &c->d_CS, (size_t)N));
  HG_CUDA(c, dalloc(c, &c->d_inletQ, std::max<size_t>(c->inletQ.size(), 1)));
  HG_CUDA(c, dalloc(c, &c->d_exitWse, std::max<size_t>(c->exitWse.size(), 1)));
  HG_CUDA(c, dalloc(c, &c->d_totalA, std::max<size_t>(c->inletQ.size(), 1)));
  // the FP32 unfused conveyance totals' blocks per group (k_inlet_total_f32)
  size_t inletMost = 1;
  for (size_t g = 0; g + 1 < inletOff.size(); ++g)
    inletMost = std::max<size_t>(inletMost, (size_t)(inletOff[g + 1] - inletOff[g]));
  const int32_t inletParts = (int32_t)((inletMost + kStageBlockF32 - 1) / kStageBlockF32);
  double* d_inletPart = nullptr;
  unsigned int* d_inletTicket = nullptr;
  {
    const size_t groups = std::max<size_t>(c->inletQ.size(), 1);
    HG_CUDA(c, dalloc(c, &d_inletPart, groups * (size_t)inletParts));
    HG_CUDA(c, dalloc(c, &d_inletTicket, groups));
    HG_CUDA(c, cudaMemsetAsync(d_inletTicket, 0, groups * sizeof(unsigned int), c->stream));
  }
  HG_CUDA(c, dalloc(c, &c->d_perm, (size_t)N));
  HG_CUDA(c, dalloc(c, &c->Quser, (size_t)3 * N));
  HG_CUDA(c, dalloc(c, &c->QB, (size_t)3 * N));   // FP64 stage buffer; also the FP32 path's RHS output
  if (c->precision == HG_FP64) {
    HG_CUDA(c, dalloc(c, &c->QA, (size_t)3 * N));
  } else {
    HG_CUDA(c, dalloc(c, &c->XA, (size_t)N));
    HG_CUDA(c, dalloc(c, &c->XB, (size_t)N));
    HG_CUDA(c, dalloc(c, &c->XQA, (size_t)N));
    HG_CUDA(c, dalloc(c, &c->XQB, (size_t)N));
  }
  // Scalars
  HG_CUDA(c, dalloc(c, &c->ds.dt, 1));
  HG_CUDA(c, dalloc(c, &c->ds.dtf, 1));
  HG_CUDA(c, dalloc(c, &c->ds.cflMin, 2));
  HG_CUDA(c, dalloc(c, &c->ds.cflMinF, 2));
  HG_CUDA(c, dalloc(c, &c->ds.stepIdx, 1));
  HG_CUDA(c, dalloc(c, &c->ds.tSum, 1));
  HG_CUDA(c, dalloc(c, &c->ds.flags, 1));
  c->ds.dtMin = kDtMinDefault;
  // Ensembles: every member takes its own step.  Each member's cells form one
  // contiguous range in the device order (the orderings keep members apart),
  // at the member's offset of the caller order.
  if (c->memberCellOff.size() >= 2) {
    const int M = (int)c->memberCellOff.size() - 1;
    for (int mm = 0; mm < M; ++mm)
      for (int i = c->memberCellOff[mm]; i < c->memberCellOff[mm + 1]; ++i)
        if (c->perm[i] < c->memberCellOff[mm] || c->perm[i] >= c->memberCellOff[mm + 1])
          return fail(c, HG_ERR_MESH, "ensemble: a member's cells are not contiguous in the device order");
    std::vector<int32_t> inletMember(std::max<size_t>(inletCell.empty() ? 0 : m.inletGroups.size(), 1), 0);
    for (int mm = 0; mm < M; ++mm)
      for (int g = c->memberInletOff[mm]; g < c->memberInletOff[mm + 1]; ++g) inletMember[g] = mm;
    std::vector<int32_t> memberOf((size_t)N);
    for (int mm = 0; mm < M; ++mm)
      for (int i = c->memberCellOff[mm]; i < c->memberCellOff[mm + 1]; ++i) memberOf[i] = mm;
    int32_t *dOff = nullptr, *dInM = nullptr, *dOf = nullptr;
    HG_CUDA(c, dalloc(c, &dOff, (size_t)M + 1));
    HG_CUDA(c, dalloc(c, &dInM, inletMember.size()));
    HG_CUDA(c, dalloc(c, &dOf, (size_t)N));
    HG_CUDA(c, upload(c, dOff, c->memberCellOff));
    HG_CUDA(c, upload(c, dInM, inletMember));
    HG_CUDA(c, upload(c, dOf, memberOf));
    HG_CUDA(c, dalloc(c, &c->ds.dtM, (size_t)M));
    HG_CUDA(c, dalloc(c, &c->ds.dtMf, (size_t)M));
    HG_CUDA(c, dalloc(c, &c->ds.tM, (size_t)M));
    HG_CUDA(c, dalloc(c, &c->ds.cflMinM, (size_t)M));
    HG_CUDA(c, dalloc(c, &c->ds.cflMinMF, (size_t)M));
    c->ds.memberOff = dOff;
    c->ds.memberOfCell = dOf;
    c->ds.inletMember = dInM;
    c->ds.nMembers = M;
    HG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  HG_CUDA(c, dalloc(c, &c->d_tot, (size_t)2 * kMaxFusedInlets));
  // Fused FP32 stepping: the stage blocks holding inlet-Q cells, numbered in block order.
  std::vector<int32_t> blockSlot;
  {
    DevMesh sized;
    sized.n = N;
    const int nBlocks = std::max(stage_blocks_f32(sized), 1);
    blockSlot.assign(nBlocks, -1);
    for (int32_t cell : inletCell) blockSlot[cell / kStageBlockF32] = 0;
    c->nSlots = 0;
    c->nWarps = 0;
    for (int b = 0; b < nBlocks; ++b)
      if (blockSlot[b] == 0) {
        blockSlot[b] = c->nSlots++;
        const int cells = std::min(kStageBlockF32, N - b * kStageBlockF32);
        c->nWarps += (cells + 31) / 32;
      }
    // warp sums of the fused inlet totals; the slots of warps past the last cell stay zero
    const size_t np = (size_t)kMaxFusedInlets * std::max(c->nSlots, 1) * (kStageBlockF32 / 32);
    HG_CUDA(c, dalloc(c, &c->d_partials, np));
    HG_CUDA(c, cudaMemsetAsync(c->d_partials, 0, np * sizeof(double), c->stream));
    HG_CUDA(c, dalloc(c, &c->d_blockSlot, blockSlot.size()));
  }
  HG_CUDA(c, dalloc(c, &c->d_ticket, 1));
  HG_CUDA(c, cudaMemsetAsync(c->d_ticket, 0, sizeof(unsigned int), c->stream));
  {
    int rc = ensure_dt_capacity(c, 1024);
    if (rc) return rc;
  }
  // L2 flush buffer: 256 MB written, then a different 256 MB read (each larger than the 126 MB L2).
  c->flushBytes = (size_t)512 << 20;
  HG_CUDA(c, dalloc(c, reinterpret_cast<char**>(&c->flushBuf), c->flushBytes));

  // FP32 slot records {nx, ny, L, nb as bits}
  std::vector<float4> SL(nb.size());
  for (size_t i = 0; i < nb.size(); ++i) {
    float4 r;
    r.x = (float)snx[i];
    r.y = (float)sny[i];
    r.z = (float)slen[i];
    std::memcpy(&r.w, &nb[i], sizeof(float));
    SL[i] = r;
  }
  // Pipelined stage tables (degree <= 4): per tile of kStageBlockF32 cells, the
  // out-of-tile neighbours in order of first reference, and the slot records
  // with tile-local neighbour indices.
  std::vector<float4> SLp;
  std::vector<int32_t> halo;
  if (S <= 4) {
    const int nTiles = (N + kStageBlockF32 - 1) / kStageBlockF32;
    SLp = SL;
    halo.assign((size_t)nTiles * kHaloMax, -1);
    std::vector<int32_t> seen(N, -1);   // cell -> halo slot in the current tile
    bool fits = true;
    for (int t = 0; t < nTiles && fits; ++t) {
      const int c0 = t * kStageBlockF32, c1 = std::min(N, c0 + kStageBlockF32);
      int h = 0;
      for (int cell = c0; cell < c1 && fits; ++cell)
        for (int k = 0; k < S; ++k) {
          const size_t i = (size_t)k * N + cell;
          const int32_t v = nb[i];
          if (v < 0) continue;
          int32_t loc;
          if (v >= c0 && v < c1) {
            loc = v - c0;
          } else {
            if (seen[v] < 0 || halo[(size_t)t * kHaloMax + seen[v]] != v) {
              if (h == kHaloMax) { fits = false; break; }
              seen[v] = h;
              halo[(size_t)t * kHaloMax + h] = v;
              ++h;
            }
            loc = kStageBlockF32 + seen[v];
          }
          std::memcpy(&SLp[i].w, &loc, sizeof(float));
        }
    }
    if (!fits) {
      SLp.clear();
      halo.clear();
    }
  }
  float4* d_SLp = nullptr;
  int32_t* d_halo = nullptr;
  if (!SLp.empty()) {
    HG_CUDA(c, dalloc(c, &d_SLp, SLp.size()));
    HG_CUDA(c, dalloc(c, &d_halo, halo.size()));
    HG_CUDA(c, upload(c, d_SLp, SLp));
    HG_CUDA(c, upload(c, d_halo, halo));
  }
  // Face-once stage tables (need the halo tables)
  std::vector<float4> FL;
  std::vector<int32_t> FLoff;
  std::vector<uint2> FR;
  int32_t faceMax = 0;
  float4* d_FL = nullptr;
  int32_t* d_FLoff = nullptr;
  uint2* d_FR = nullptr;
  if (!SLp.empty() && build_face_tables(N, S, nbf, nb, SL, SLp, FL, FLoff, FR, faceMax)) {
    HG_CUDA(c, dalloc(c, &d_FL, FL.size()));
    HG_CUDA(c, dalloc(c, &d_FLoff, FLoff.size()));
    HG_CUDA(c, dalloc(c, &d_FR, FR.size()));
    HG_CUDA(c, upload(c, d_FL, FL));
    HG_CUDA(c, upload(c, d_FLoff, FLoff));
    HG_CUDA(c, upload(c, d_FR, FR));
  }
  c->h_area = to_float(area);
  HG_CUDA(c, upload(c, d_nb, nb));
  HG_CUDA(c, upload(c, c->d_blockSlot, blockSlot));
  HG_CUDA(c, upload(c, d_snx, snx));
  HG_CUDA(c, upload(c, d_sny, sny));
  HG_CUDA(c, upload(c, d_slen, slen));
  HG_CUDA(c, upload(c, d_SL, SL));
  std::vector<float> lp23f = to_float(bfLp23);
  HG_CUDA(c, upload(c, d_area, area));
  HG_CUDA(c, upload(c, d_bfInfo, bfInfo));
  HG_CUDA(c, upload(c, d_lp23, bfLp23));
  HG_CUDA(c, upload(c, d_lp23f, lp23f));
  HG_CUDA(c, upload(c, d_bflp53, bfLp53));
  HG_CUDA(c, upload(c, d_inletOff, inletOff));
  HG_CUDA(c, upload(c, d_inletCell, inletCell));
  HG_CUDA(c, upload(c, d_lp53, inletLp53));
  std::vector<int32_t> permv(c->perm.begin(), c->perm.end());
  HG_CUDA(c, upload(c, c->d_perm, permv));
  // Keep host copies alive until the async copies finish.
  HG_CUDA(c, cudaStreamSynchronize(c->stream));

  DevMesh& dm = c->dm;
  dm.n = N;
  dm.nslot = S;
  dm.nbf = nbf;
  dm.nInlet = (int32_t)m.inletGroups.size();
  dm.nExit = (int32_t)m.exitGroups.size();
  dm.nb = d_nb; dm.snx = d_snx; dm.sny = d_sny; dm.slen = d_slen;
  dm.SL = d_SL;
  dm.SLp = d_SLp;
  dm.halo = d_halo;
  dm.FL = d_FL;
  dm.FLoff = d_FLoff;
  dm.FR = d_FR;
  dm.faceMax = d_FL ? faceMax : 0;
  dm.stageKernel = d_SLp ? kStagePipe : kStageGather;
  // The autotuner's family (see autotune_stage): HG_STAGE_FAMILY=gather|face, else kDefaultFamily
  {
    const char* e = std::getenv("HG_STAGE_FAMILY");
    int fam = kDefaultFamily;
    if (e && std::strcmp(e, "gather") == 0) fam = 0;
    if (e && std::strcmp(e, "face") == 0) fam = 1;
    c->stageFamily = (fam == 1 && d_FL) ? 1 : 0;
    if (c->stageFamily == 1) dm.stageKernel = kStageFace;
    // the mesh signature of the autotune cache: the device-order face tables
    uint64_t h = fnv1a(nb.data(), nb.size() * sizeof(int32_t));
    h = fnv1a(SL.data(), SL.size() * sizeof(float4), h);
    c->meshSig = h;
  }
  dm.bfInfo = d_bfInfo; dm.bfLp23 = d_lp23; dm.bfLp23f = d_lp23f; dm.bfLp53 = d_bflp53;
  dm.bfExitRel = c->d_bfExitRel;
  dm.inletOff = d_inletOff; dm.inletCell = d_inletCell; dm.inletLp53 = d_lp53;
  dm.area = d_area; dm.hst = c->d_hst; dm.zb = c->d_zb; dm.man = c->d_man; dm.s0x = c->d_s0x; dm.s0y = c->d_s0y;
  dm.CP = c->d_CP; dm.CS = c->d_CS;
  dm.exitWse = c->d_exitWse; dm.inletQ = c->d_inletQ; dm.totalA = c->d_totalA;
  dm.inletPart = d_inletPart; dm.inletTicket = d_inletTicket; dm.inletParts = inletParts;
  dm.g = c->k.g; dm.kn2 = c->k.k_n * c->k.k_n; dm.hsm = c->k.h_small;
  dm.gf = (float)c->k.g; dm.kn2f = (float)(c->k.k_n * c->k.k_n); dm.hsmf = (float)c->k.h_small;
  dm.hsmLo = (float)(c->k.h_small - (double)dm.hsmf);
  dm.riemann = c->k.riemann;
  c->slotNb = d_nb;
  int rc = upload_cells(c);
  if (rc) return rc;
  rc = upload_boundary_values(c);
  if (rc) return rc;
  launch_reset_scalars(c->ds, c->stream);
  HG_CUDA(c, cudaStreamSynchronize(c->stream));
  HG_CUDA(c, cudaGetLastError());
  return HG_OK;
}
