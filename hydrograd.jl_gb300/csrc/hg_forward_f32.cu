// FP32-compensated stage kernels, step bookkeeping and renumbering kernels.
//
// One fused pass per explicit stage.  Each thread owns one cell (device order)
// and gathers its faces in the reference's local order (compute_inviscid_fluxes,
// src/fvm/discretization/semi_discretize_swe_2D.jl:286-419): clamp, ghost
// state, Roe flux, -sum F L / A, Manning friction + bed-slope source, then the
// compensated stage update and the depth-positivity clamp.  Gather form: no
// atomics; per-cell summation order fixed, so results are bit-reproducible.
// Cell records are packed (hg_f32.cuh) so that a cell costs a few 16-byte
// loads, and the slot loop is unrolled to the mesh's maximum cell degree so
// that all of a cell's slot and neighbour loads are in flight together.
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "hg_async.cuh"
#include "hg_device.cuh"
#include "hg_f32.cuh"
#include "hg_members.cuh"
#include "hg_pdl.cuh"
#include "hg_reduce.cuh"
#include "hg_resfn.cuh"
#include "hg_state.hpp"
#include "hg_tma.cuh"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = kStageBlockF32;

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

// Flux F (times nothing: the caller scales by the face length) of slot sl of
// the cell with side L, own quantities own.  LOC: the slot's neighbour word
// holds a tile-local index (bits 0-8: own cells at [0, kBlock) of sX / sP,
// halo cells at [kBlock, ...) of hX / hP); otherwise a cell id.  RS: the
// Riemann solver fixed at compile time (kRiemannRoe / kRiemannHll), or -1 for
// the context's at run time (DevMesh::riemann).
// TB: the cells of the launch's block (the non-LOC in-block test; kBlock
// unless the gather kernel runs another tile size).
template <bool LOC, int RS, int TB = kBlock>
__device__ __forceinline__ void one_face_f32(const DevMesh& m, const float4* __restrict__ X, const float4* sX,
                                             const float4* sP, const float4* hX, const float4* hP, int base, int c,
                                             const SideF32& L, const OwnF32& own, float2 hstPair, float4 sl, int32_t nb,
                                             const double* __restrict__ totalA, float man, int32_t* flags,
                                             float F[3]) {
  const float nx = sl.x, ny = sl.y;
  Side<float> R;
  float dxi, dhst = 0.0f;
  int bank = -1;   // the wall test of a face with one dry side, in FP64 (bank_wall_f64)
  if (nb >= 0) {
    float4 xr, pr;
    if constexpr (LOC) {
      const int li = nb & 511;
      if (li < kBlock) {
        xr = sX[li];
        pr = sP[li];
      } else {
        xr = hX[li - kBlock];
        pr = hP[li - kBlock];
      }
    } else {
      const unsigned int ln = (unsigned int)(nb - base);   // in-block neighbour: staged record
      if (ln < (unsigned int)TB) {
        xr = sX[ln];
        pr = sP[ln];
      } else {
        xr = __ldg(&X[nb]);
        pr = __ldg(&m.CP[nb]);
      }
    }
    const SideF32 r = make_side_f32(xr, pr, m.hsmf, m.hsmLo);
    R = r.s;
    dxi = (r.s.xi - L.s.xi) + (r.xlo - L.xlo);
    dhst = (pr.x - hstPair.x) + (pr.y - hstPair.y);   // hstill_R - hstill_L from the pairs
    if (L.s.dry != r.s.dry) {   // a front face
      int g = nb;               // the neighbour's cell id
      if constexpr (LOC) {
        const int li = nb & 511;
        g = li < kBlock ? base + li : __ldg(&m.halo[(size_t)(base / kBlock) * kHaloMax + (li - kBlock)]);
      }
      bank = L.s.dry ? bank_wall_f64(m, r.s.xi, r.xlo, g, c) : bank_wall_f64(m, L.s.xi, L.xlo, c, g);
    }
  } else {
    const int32_t bf = boundary_index(nb);
    const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
    if (type == kBcInletQ && !(totalA[grp] > 1e-10)) atomicOr(flags, 2);   // bc_2D.jl:679
    R = ghost_state<float>(L.s, type, nx, ny, m.hsmf, type == kBcExitH ? (float)m.exitWse[grp] : 0.0f,
                           type == kBcInletQ ? (float)m.inletQ[grp] : 0.0f,
                           type == kBcInletQ ? (float)totalA[grp] : 1.0f, m.bfLp23f[bf], man);
    // xi_ghost - xi = (h_ghost - h) + ((h - hstill) - xi); for a wet exit-H
    // ghost, from (WSE - zb) - hstill formed in FP64
    dxi = (R.h - L.s.h) + L.excess;
    if (type == kBcExitH && !R.dry) dxi = m.bfExitRel[bf] - (L.s.xi + L.xlo);
    if (type == kBcExitH && L.s.dry != R.dry)   // (the other ghosts are as wet as their cell)
      bank = L.s.dry ? bank_exit_f64(m, grp, c) : bank_wall_f64(m, L.s.xi, L.xlo, c, c);
  }
  const int rs = RS >= 0 ? RS : m.riemann;
  if (!L.s.dry && !R.dry) {
    if (rs == kRiemannHll) hll_flux_wet_f32(L.s, own, R, dxi, dhst, m.gf, nx, ny, F);
    else roe_flux_wet_f32(L.s, own, R, dxi, dhst, m.gf, nx, ny, F);
  } else {
    riemann_flux<float>(rs, L.s, R, dxi, m.gf, nx, ny, m.hsmf, F, bank);
    F[1] -= own.p * nx;   // the own pressure shift (pressure_jump_f32)
    F[2] -= own.p * ny;
  }
}

template <int NS, bool LOC, int RS, int TB = kBlock>
__device__ __forceinline__ void face_sum_f32(const DevMesh& m, const float4* __restrict__ X, const float4* sX,
                                             const float4* sP, const float4* hX, const float4* hP, int base, int c,
                                             const SideF32& L, const OwnF32& own, float2 hstPair,
                                             const float4 (&sl)[NS], const double* __restrict__ totalA, float man,
                                             int32_t* flags, float& f0, float& f1, float& f2) {
  f0 = 0.0f; f1 = 0.0f; f2 = 0.0f;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const int32_t nb = slot_nb(sl[k]);
    if (nb == kNoFace) continue;
    float F[3];
    one_face_f32<LOC, RS, TB>(m, X, sX, sP, hX, hP, base, c, L, own, hstPair, sl[k], nb, totalA, man, flags, F);
    const float len = sl[k].z;
    f0 = fmaf(F[0], len, f0);
    const float2 f12 = fma2(p2(F[1], F[2]), p2(len), p2(f1, f2));
    f1 = f12.x;
    f2 = f12.y;
  }
}

template <int NS>
__device__ __forceinline__ float cfl_candidate_f32(const DevMesh& m, const float4 (&sl)[NS], float h, float qx,
                                                   float qy, bool dry, float area) {
  if (dry) { qx = 0.0f; qy = 0.0f; }
  const float u = qx / h, v = qy / h, a = sqrtf(m.gf * h);
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (slot_nb(sl[k]) == kNoFace) continue;
    s += sl[k].z * (fabsf(u * sl[k].x + v * sl[k].y) + a);
  }
  return area / s;
}

template <int NS>
__device__ __forceinline__ void load_slots(const DevMesh& m, int c, float4 (&sl)[NS]) {
#pragma unroll
  for (int k = 0; k < NS; ++k) sl[k] = __ldg(&m.SL[(size_t)k * m.n + c]);
}

// Inlet-Q conveyance totals of a fused stage's output state (bc_2D.jl:673-676).
// The sums are keyed to fixed tiles of kBlock cells, whatever the launch's
// block size: each warp of a tile holding inlet cells writes its warp sum
// (partials[g][slot][warp]), and the last warp to arrive adds them -- each
// tile's warp sums in the fixed tree of devred::block_sum (halves folded), the
// tiles' sums lane-strided and folded across the warp -- so every stage
// kernel and tile size forms the same totals.  Warps past the last cell never
// write: their partials stay at the zeros the buffer was allocated with.
// Only the warps of those few tiles reload the slot records, so the others
// carry no extra registers for it.
constexpr int kTileWarps = kBlock / 32;

// Manning's n of a cell from its clamped side state, for the n(h, Umag, ks)
// functions (ResDev kinds power law .. h_Umag_ks) evaluated in the fused
// stages (RESFN) instead of a separate resistance pass: as k_res_cells forms
// it, Umag = |q| / h of the clamped state.
__device__ __forceinline__ float own_manning_f32(const DevMesh& m, const Side<float>& s, int c) {
  const float u = s.hu / s.h, v = s.hv / s.h;
  return manning_fn<float>(m.res, s.h, sqrtf(u * u + v * v), m.res.ks ? (float)m.res.ks[c] : 0.0f);
}

// RESFN: n of the output state from the function (Xo: the output records),
// not the resident CP.w.
template <int NS, bool RESFN = false>
__device__ __forceinline__ void fused_inlet_totals(const DevMesh& m, const StageFuse& f, int c, float hOut,
                                                   bool wetOut, const float4* Xo = nullptr) {
  const int lane = threadIdx.x & 31;
  const int c0 = c - lane;   // the warp's first cell; warps never straddle tiles (32 divides kBlock)
  if (c0 >= m.n) return;     // uniform over the warp
  const int slot = f.blockSlot[c0 / kBlock];
  if (slot < 0) return;
  const int wIdx = (c0 % kBlock) / 32;
  const int ng = m.nInlet;
  float nOut = 0.0f;
  if (wetOut) {
    if constexpr (RESFN) nOut = own_manning_f32(m, make_side_f32(Xo[c], m.CP[c], m.hsmf, m.hsmLo).s, c);
    else nOut = m.CP[c].w;
  }
  for (int g = 0; g < ng; ++g) {
    double v = 0.0;
    if (wetOut) {
      for (int k = 0; k < NS; ++k) {
        const int32_t nb = slot_nb(m.SL[(size_t)k * m.n + c]);
        if (nb >= 0 || nb == kNoFace) continue;
        const int32_t bf = boundary_index(nb);
        if (m.bfInfo[bf] == (kBcInletQ | (g << 2))) v += m.bfLp53[bf] * (double)hOut / (double)nOut;
      }
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) f.partials[((size_t)g * f.nSlots + slot) * kTileWarps + wIdx] = v;
  }
  unsigned int last = 0u;
  if (lane == 0) {
    __threadfence();
    last = atomicAdd(f.ticket, 1u) == (unsigned int)f.nWarps - 1u ? 1u : 0u;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();
  for (int g = 0; g < ng; ++g) {
    double acc = 0.0;
    for (int b = lane; b < f.nSlots; b += 32) {
      const double* p = f.partials + ((size_t)g * f.nSlots + b) * kTileWarps;
      double r[kTileWarps];
#pragma unroll
      for (int i = 0; i < kTileWarps; ++i) r[i] = __ldcg(&p[i]);
#pragma unroll
      for (int h = kTileWarps / 2; h >= 1; h >>= 1)
#pragma unroll
        for (int i = 0; i < h; ++i) r[i] += r[i + h];
      acc += r[0];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) f.totalOut[g] = acc;
  }
  if (lane == 0) *f.ticket = 0u;
}

// dt of a fused step: from the published CFL minimum (CFL mode) or the fixed dt.
__device__ __forceinline__ double fused_dt(const DevScalars& s, const StageFuse& f) {
  if (!f.cflMode) return *s.dt;
  const double mn = fmin(__longlong_as_double((long long)s.cflMin[f.parity]),
                         (double)__uint_as_float(s.cflMinF[f.parity]));
  return f.cfl * mn;
}

// The stage kernel is latency-bound (neighbour gathers): for meshes of degree
// <= 4 it is held to the register budget of HG_STAGE_MIN_BLOCKS resident
// blocks per SM (by default 64 registers a thread, no spills; 50% occupancy).
#ifndef HG_STAGE_MIN_BLOCKS
#define HG_STAGE_MIN_BLOCKS (1024 / kBlock)
#endif
template <int NS>
constexpr int stage_min_blocks() { return NS <= 4 ? HG_STAGE_MIN_BLOCKS : 1; }

template <int NS, int MODE>
__device__ __forceinline__ void stage_finish(const DevMesh& m, const DevScalars& s, const SideF32& L, float f0,
                                             float f1, float f2, int c, const float4 (&sl)[NS], float4 xin, float4 cp,
                                             float4 cs, const float2* qinP, const float4* xbP, const float2* qbP,
                                             int k, float dt, StateF32 Xout, double* Rout, bool cfl, float& cand,
                                             float& hOut, bool& wetOut);

// One cell of a stage: clamp, faces, sources, compensated update and clamp of
// the output, CFL candidate.  sX / sP hold the records of cells [base, base +
// kBlock) for in-block neighbours.  The input state's lo parts and (stage 2)
// the base state are read at qinP[k], xbP[k], qbP[k] -- global arrays (k = c)
// or a tile staged in shared memory -- where they are used.
template <int NS, int MODE, bool LOC = false, int RS = -1, int TB = kBlock, bool RESFN = false>
__device__ __forceinline__ void stage_cell(const DevMesh& m, const DevScalars& s, const float4* __restrict__ X,
                                           const float4* sX, const float4* sP, const float4* hX, const float4* hP,
                                           int base, int c,
                                           const float4 (&sl)[NS], float4 xin, float4 cp, float4 cs,
                                           const float2* qinP, const float4* xbP, const float2* qbP, int k, float dt,
                                           const double* totalIn, StateF32 Xout, double* Rout, bool cfl,
                                           float& cand, float& hOut, bool& wetOut) {
  const SideF32 L = make_side_f32(xin, cp, m.hsmf, m.hsmLo);
  const OwnF32 own = own_f32(L.s, m.gf);
  float4 cpn = cp;   // RESFN: the cell's n from its own state, for the friction and the inlet ghost
  if constexpr (RESFN) cpn.w = own_manning_f32(m, L.s, c);
  float f0, f1, f2;
  face_sum_f32<NS, LOC, RS, TB>(m, X, sX, sP, hX, hP, base, c, L, own, make_float2(cp.x, cp.y), sl, totalIn, cpn.w, s.flags, f0, f1, f2);
  stage_finish<NS, MODE>(m, s, L, f0, f1, f2, c, sl, xin, cpn, cs, qinP, xbP, qbP, k, dt, Xout, Rout, cfl, cand, hOut,
                         wetOut);
}

// The rest of a cell's stage once its face sums f0..f2 (sum_k F_k L_k) are
// formed: sources, -sum / A, compensated update, clamp of the output, CFL
// candidate (or, in RHS mode, the RHS).
template <int NS, int MODE>
__device__ __forceinline__ void stage_finish(const DevMesh& m, const DevScalars& s, const SideF32& L, float f0,
                                             float f1, float f2, int c, const float4 (&sl)[NS], float4 xin, float4 cp,
                                             float4 cs, const float2* qinP, const float4* xbP, const float2* qbP,
                                             int k, float dt, StateF32 Xout, double* Rout, bool cfl, float& cand,
                                             float& hOut, bool& wetOut) {
  const float A = cs.z;
  const float rA = -1.0f / A;
  const float r0 = f0 * rA;
  const float2 r12 = mul2(p2(f1, f2), p2(rA));
  // Manning friction, or the flow-resistance closure F q / |q|_smooth
  // (semi_discretize_swe_2D.jl:517-529) with F from the resistance kernels.
  const float fr = m.res.kind == kResUdeFlowResistance
                       ? m.res.fresF[c] / smooth_sqrt(L.s.hu * L.s.hu + L.s.hv * L.s.hv)
                       : friction_coef(m.gf, m.kn2f, m.hsmf, cp.w, L.s.h, L.s.hu, L.s.hv);
  // (h > h_small) (g xi S0 - friction q), the momentum rows as one pair
  const float2 src = L.s.dry ? p2(0.0f) : fma2(p2(m.gf * L.s.xi), p2(cs.x, cs.y), mul2(p2(-fr), p2(L.s.hu, L.s.hv)));
  const float d0 = r0;
  const float2 d12 = add2(r12, src);
  if constexpr (MODE == kModeRhs) {
    Rout[c] = d0; Rout[m.n + c] = d12.x; Rout[2 * m.n + c] = d12.y;
  } else if constexpr (MODE == kModeRhsF32) {
    float* R = reinterpret_cast<float*>(Rout);
    R[c] = d0; R[m.n + c] = d12.x; R[2 * m.n + c] = d12.y;
  } else {
    const float2 qin = qinP[k];
    const float inc0 = dt * d0;
    const float2 inc12 = mul2(p2(dt), d12);
    float xh[3], xl[3];
    float2 qh, ql;
    if constexpr (MODE == kModeStage2) {
      const float4 xb = xbP[k];
      const float2 qb = qbP[k];
      float sh, slo;
      df_add2(xb.x, xb.y, xin.x, xin.y, sh, slo);
      df_add(sh, slo, inc0, xh[0], xl[0]);
      xh[0] *= 0.5f;
      xl[0] *= 0.5f;
      float2 sh2, sl2;
      df_add2_2(p2(xb.z, xb.w), qb, p2(xin.z, xin.w), qin, sh2, sl2);
      df_add_2(sh2, sl2, inc12, qh, ql);
      qh = mul2(qh, p2(0.5f));
      ql = mul2(ql, p2(0.5f));
    } else {
      df_add(xin.x, xin.y, inc0, xh[0], xl[0]);
      df_add_2(p2(xin.z, xin.w), qin, inc12, qh, ql);
    }
    xh[1] = qh.x; xh[2] = qh.y;
    xl[1] = ql.x; xl[2] = ql.y;
    DepthF32 dn = depth_f32(xh[0], xl[0], cp.x, cp.y, m.hsmf, m.hsmLo);
    bool clamp = dn.dry;   // h <= h_small (pair granularity): h = h_small, q = 0
    if constexpr (MODE == kModeEulerRef) clamp = (double)xh[0] + (double)xl[0] < m.hsm;
    if (clamp) {
      const double x0 = (MODE == kModeEulerRef) ? m.hsm : dry_xi(m.hsm, (double)cp.x + (double)cp.y);
      xh[0] = (float)x0;
      xl[0] = (float)(x0 - (double)xh[0]);
      xh[1] = xl[1] = xh[2] = xl[2] = 0.0f;
      dn.dry = true;
      dn.h = m.hsmf;
    }
    if (!(isfinite(xh[0]) && isfinite(xh[1]) && isfinite(xh[2]))) atomicOr(s.flags, 1);
    Xout.x[c] = make_float4(xh[0], xl[0], xh[1], xh[2]);
    Xout.q[c] = make_float2(xl[1], xl[2]);
    if (cfl) cand = fminf(cand, cfl_candidate_f32<NS>(m, sl, dn.h, xh[1], xh[2], dn.dry, A));
    hOut = dn.h;
    wetOut = !dn.dry;
  }
}

// Step bookkeeping of a fused stage 1 (block 0, thread 0), and clearing of
// the CFL buffer stage 2 publishes into.
__device__ __forceinline__ void fused_record(const DevScalars& s, const StageFuse& f) {
  const double dt = fused_dt(s, f);
  if (f.cflMode && !(dt >= s.dtMin)) atomicOr(s.flags, 8);   // the step collapsed (or is NaN)
  const int k = *s.stepIdx;
  if (k < s.dtCap) s.dtHist[k] = dt;
  *s.stepIdx = k + 1;
  *s.tSum += dt;
  *s.dt = dt;
  *s.dtf = (float)dt;
  s.cflMin[1 - f.parity] = (unsigned long long)__double_as_longlong(INFINITY);
  s.cflMinF[1 - f.parity] = __float_as_uint(INFINITY);
}

// GB300 issues FP64 at a small fraction of the FP32 rate, so the per-cell path
// holds no FP64 arithmetic: the stage mode is a template parameter (the FP64
// comparison of the reference Euler clamp exists only in that instance), and
// the fused step's dt is formed once per block.
// MINB > 0: the register budget of MINB resident blocks per SM (a shape the
// autotuner chooses among; the arithmetic does not depend on it).
// TB: cells per block (the autotuner's tile-size candidates: 128, 256, 512;
// a cell's arithmetic does not depend on it).
// RESFN: Manning's n from an n(h, Umag, ks) function of the state, evaluated
// here (DevMesh::res) instead of read from CP.w.
template <int NS, bool FUSED, int MODE, int RS = -1, int MINB = 0, int TB = kBlock, bool RESFN = false>
__global__ void __launch_bounds__(TB, MINB > 0 ? MINB : stage_min_blocks<NS>())
    k_stage_f32(DevMesh m, DevScalars s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, double* Rout, int cfl,
                StageFuse f) {
  pdl_enter();
  const int base = blockIdx.x * TB;
  const int c = base + threadIdx.x;
  const bool active = c < m.n;
  float cand = INFINITY;
  float hOut = 0.0f;      // output depth, and whether the output cell is wet (fused inlet totals)
  bool wetOut = false;
  // The block's own state and parameter records, staged for the neighbours in
  // the block (most of them, in Hilbert order): every global load of the block
  // is issued before the barrier, and in-block neighbour reads skip a second
  // round trip to L2/DRAM.
  __shared__ float4 sX[TB], sP[TB];
  __shared__ float dtShared;
  float4 sl[NS], xin, cp, cs;
  if (active) {
    load_slots<NS>(m, c, sl);
    xin = __ldg(&Xin.x[c]);
    cp = __ldg(&m.CP[c]);
    cs = __ldg(&m.CS[c]);
    sX[threadIdx.x] = xin;
    sP[threadIdx.x] = cp;
  }
  if constexpr (FUSED) {
    if (threadIdx.x == 0) dtShared = (float)fused_dt(s, f);
  }
  __syncthreads();
  const int mem = (!FUSED && s.nMembers > 0 && active) ? member_of(s, c) : -1;   // an ensemble member's own step
  if (active) {
    const float dt = (MODE == kModeRhs || MODE == kModeRhsF32) ? 0.0f
                                                               : (FUSED ? dtShared : (mem >= 0 ? s.dtMf[mem] : *s.dtf));
    stage_cell<NS, MODE, false, RS, TB, RESFN>(m, s, Xin.x, sX, sP, nullptr, nullptr, base, c, sl, xin, cp, cs, Xin.q, Xbase.x,
                                     Xbase.q, c,
                         dt, FUSED ? f.totalIn : m.totalA, Xout, Rout, cfl, cand, hOut, wetOut);
  }
  if (FUSED && f.record && blockIdx.x == 0 && threadIdx.x == 0) fused_record(s, f);
  if (cfl && !FUSED && s.nMembers > 0) member_min_publish_f(s, cand, mem);
  else if (cfl) block_min_publish_f(cand, FUSED ? s.cflMinF + (1 - f.parity) : s.cflMinF);
  if (FUSED && m.nInlet > 0) fused_inlet_totals<NS, RESFN>(m, f, c, hOut, wetOut, Xout.x);
}

// ---------------------------------------------------------------------------
// Persistent fused stage with TMA tile prefetch
// ---------------------------------------------------------------------------
// Each CTA walks the 256-cell tiles t = blockIdx.x, + gridDim.x, ...  While it
// computes tile t from shared memory, bulk copies (cp.async.bulk, one per
// array: the NS slot records, X, CP, CS, XQ, and in stage 2 the base state)
// bring tile t + gridDim.x into the other of two buffers, completing on that
// buffer's mbarrier -- so the own-cell data of a tile is on chip before its
// threads start, and only out-of-tile neighbours are gathered from L2/DRAM.
// A partial last tile is loaded with plain loads.  Results equal k_stage_f32's
// (same stage_cell, same block = tile decomposition for the inlet partials).
constexpr int kTmaCtasPerSm = 3;

template <int NS, int MODE>
struct TmaTile {
  static constexpr uint32_t kRec = kBlock * sizeof(float4);   // 4096 B
  static constexpr uint32_t kLo = kBlock * sizeof(float2);    // 2048 B
  static constexpr uint32_t kSL = 0, kX = NS * kRec, kCP = kX + kRec, kCS = kCP + kRec, kQ = kCS + kRec;
  static constexpr uint32_t kXB = kQ + kLo, kQB = kXB + kRec;
  static constexpr uint32_t kBytes = (MODE == kModeStage2) ? kQB + kLo : kQ + kLo;   // copied per tile
  static constexpr uint32_t kBuf = (kBytes + 127u) & ~127u;
  static constexpr uint32_t kSmem = 2 * kBuf + 2 * sizeof(uint64_t);
};

template <int NS, int MODE>
__device__ __forceinline__ void tma_issue_tile(const DevMesh& m, StateF32 Xin, StateF32 Xbase, int t, unsigned char* B,
                                               uint64_t* bar) {
  using T = TmaTile<NS, MODE>;
  const size_t c0 = (size_t)t * kBlock;
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(bar, T::kBytes);
#pragma unroll
  for (int k = 0; k < NS; ++k) bulk_copy_g2s(B + T::kSL + k * T::kRec, m.SL + (size_t)k * m.n + c0, T::kRec, bar);
  bulk_copy_g2s(B + T::kX, Xin.x + c0, T::kRec, bar);
  bulk_copy_g2s(B + T::kCP, m.CP + c0, T::kRec, bar);
  bulk_copy_g2s(B + T::kCS, m.CS + c0, T::kRec, bar);
  bulk_copy_g2s(B + T::kQ, Xin.q + c0, T::kLo, bar);
  if constexpr (MODE == kModeStage2) {
    bulk_copy_g2s(B + T::kXB, Xbase.x + c0, T::kRec, bar);
    bulk_copy_g2s(B + T::kQB, Xbase.q + c0, T::kLo, bar);
  }
}

template <int NS, int MODE, int RS>
__global__ void __launch_bounds__(kBlock, kTmaCtasPerSm)
    k_stage_tma_f32(DevMesh m, DevScalars s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl, StageFuse f) {
  pdl_enter();
  using T = TmaTile<NS, MODE>;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * T::kBuf);
  __shared__ float dtShared;
  const int n = m.n;
  const int nTiles = (n + kBlock - 1) / kBlock, nFull = n / kBlock;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    dtShared = (float)fused_dt(s, f);
  }
  __syncthreads();
  int t = blockIdx.x;
  if (tid == 0 && t < nFull) tma_issue_tile<NS, MODE>(m, Xin, Xbase, t, smem, &bar[0]);
  const float dt = dtShared;
  float cand = INFINITY;
  uint32_t phases = 0u;   // bit b: parity of buffer b's next phase
  int b = 0;
  for (; t < nTiles; t += gridDim.x, b ^= 1) {
    const int tn = t + gridDim.x;
    if (tid == 0 && tn < nFull) tma_issue_tile<NS, MODE>(m, Xin, Xbase, tn, smem + (b ^ 1) * T::kBuf, &bar[b ^ 1]);
    unsigned char* B = smem + b * T::kBuf;
    const float4* bSL = reinterpret_cast<const float4*>(B + T::kSL);
    float4* bX = reinterpret_cast<float4*>(B + T::kX);
    float4* bCP = reinterpret_cast<float4*>(B + T::kCP);
    float4* bCS = reinterpret_cast<float4*>(B + T::kCS);
    float2* bQ = reinterpret_cast<float2*>(B + T::kQ);
    float4* bXB = reinterpret_cast<float4*>(B + T::kXB);
    float2* bQB = reinterpret_cast<float2*>(B + T::kQB);
    const int base = t * kBlock, c = base + tid;
    if (t < nFull) {
      const bool ok = mbar_wait(&bar[b], (phases >> b) & 1u);
      phases ^= 1u << b;
      if (!__syncthreads_and(ok)) {
        // the tile never arrived: report, let the prefetch in flight land, stop
        if (tid == 0) {
          atomicOr(s.flags, 4);
          if (tn < nFull) mbar_wait(&bar[b ^ 1], (phases >> (b ^ 1)) & 1u);
        }
        return;
      }
    } else {   // partial last tile: plain loads
      if (c < n) {
        float4* wSL = reinterpret_cast<float4*>(B + T::kSL);
#pragma unroll
        for (int k = 0; k < NS; ++k) wSL[k * kBlock + tid] = m.SL[(size_t)k * n + c];
        bX[tid] = Xin.x[c];
        bCP[tid] = m.CP[c];
        bCS[tid] = m.CS[c];
        bQ[tid] = Xin.q[c];
        if constexpr (MODE == kModeStage2) {
          bXB[tid] = Xbase.x[c];
          bQB[tid] = Xbase.q[c];
        }
      }
      __syncthreads();
    }
    float hOut = 0.0f;
    bool wetOut = false;
    if (c < n) {
      float4 sl[NS];
#pragma unroll
      for (int k = 0; k < NS; ++k) sl[k] = bSL[k * kBlock + tid];
      stage_cell<NS, MODE, false, RS>(m, s, Xin.x, bX, bCP, nullptr, nullptr, base, c, sl, bX[tid], bCP[tid], bCS[tid],
                                      bQ, bXB,
                           bQB, tid, dt, f.totalIn, Xout, nullptr, cfl, cand, hOut, wetOut);
    }
    if (m.nInlet > 0) fused_inlet_totals<NS>(m, f, c, hOut, wetOut);
    __syncthreads();   // buffer b is refilled by the copy issued at the top of the iteration after next
  }
  if (f.record && blockIdx.x == 0 && tid == 0) fused_record(s, f);
  if (cfl) block_min_publish_f(cand, s.cflMinF + (1 - f.parity));
}

// ---------------------------------------------------------------------------
// Pipelined persistent fused stage (the default for meshes of degree <= 4)
// ---------------------------------------------------------------------------
// The block-per-tile kernel pays two dependent memory latencies per tile --
// its own records, then its out-of-tile neighbours from inside the face loop
// -- and with four resident blocks per SM they leave ~40% of the issue slots
// empty.  Here each CTA walks tiles t = blockIdx.x, + gridDim.x, ... and,
// while it computes tile t, asynchronous copies (cp.async, 16 B per record,
// issued by every thread) bring tile t + gridDim.x into the other of two
// shared-memory buffers: the tile's slot records (DevMesh::SLp, neighbours as
// tile-local indices), state, parameter and source records, and its halo --
// the out-of-tile neighbour records, listed per tile on the host (DevMesh::halo).
// The halo list of the tile after that is read into a register one iteration
// ahead, so no copy waits on a load.  The compute phase then reads only shared
// memory; results equal k_stage_f32's (same stage_cell arithmetic).
constexpr int kPipeCtasPerSm = 3;

template <int NS, int MODE>
struct PipeTile {
  static constexpr uint32_t kRec = kBlock * sizeof(float4);
  static constexpr uint32_t kLo = kBlock * sizeof(float2);
  static constexpr uint32_t kHalo = kHaloMax * sizeof(float4);
  static constexpr uint32_t kSL = 0, kX = NS * kRec, kCP = kX + kRec, kCS = kCP + kRec, kQ = kCS + kRec;
  static constexpr uint32_t kHX = kQ + kLo, kHP = kHX + kHalo, kXB = kHP + kHalo, kQB = kXB + kRec;
  static constexpr uint32_t kBuf = (((MODE == kModeStage2) ? kQB + kLo : kXB) + 127u) & ~127u;
  static constexpr uint32_t kSmem = 2 * kBuf;
};

// Copies of tile t into buffer B: the thread's own cell's records, and halo
// record hid (-1: none) into halo slot threadIdx.x.
template <int NS, int MODE>
__device__ __forceinline__ void pipe_issue(const DevMesh& m, StateF32 Xin, StateF32 Xbase, int t, unsigned char* B,
                                           int hid) {
  using T = PipeTile<NS, MODE>;
  const int tid = threadIdx.x;
  const int c = t * kBlock + tid;
  if (c < m.n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) cp_async16(B + T::kSL + (k * kBlock + tid) * 16, &m.SLp[(size_t)k * m.n + c]);
    cp_async16(B + T::kX + tid * 16, &Xin.x[c]);
    cp_async16(B + T::kCP + tid * 16, &m.CP[c]);
    cp_async16(B + T::kCS + tid * 16, &m.CS[c]);
    cp_async8(B + T::kQ + tid * 8, &Xin.q[c]);
    if constexpr (MODE == kModeStage2) {
      cp_async16(B + T::kXB + tid * 16, &Xbase.x[c]);
      cp_async8(B + T::kQB + tid * 8, &Xbase.q[c]);
    }
  }
  if (hid >= 0) {
    cp_async16(B + T::kHX + tid * 16, &Xin.x[hid]);
    cp_async16(B + T::kHP + tid * 16, &m.CP[hid]);
  }
}

// FUSED: the fused step's bookkeeping (StageFuse); otherwise a plain stage of
// an unfused step (dt and inlet totals from DevScalars / DevMesh), as the
// ensembles and state-dependent resistance take.
template <int NS, int MODE, bool FUSED, int RS>
__global__ void __launch_bounds__(kBlock, kPipeCtasPerSm)
    k_stage_pipe_f32(DevMesh m, DevScalars s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl, StageFuse f) {
  pdl_enter();
  using T = PipeTile<NS, MODE>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ float dtShared;
  const int n = m.n, nTiles = (n + kBlock - 1) / kBlock, tid = threadIdx.x, G = gridDim.x;
  if (tid == 0) dtShared = FUSED ? (float)fused_dt(s, f) : *s.dtf;
  auto halo_id = [&](int t) { return (t < nTiles && tid < kHaloMax) ? m.halo[(size_t)t * kHaloMax + tid] : -1; };
  int t = blockIdx.x;
  if (t < nTiles) pipe_issue<NS, MODE>(m, Xin, Xbase, t, smem, halo_id(t));
  cp_async_commit();
  int hidNext = halo_id(t + G);
  float cand = INFINITY;
  int b = 0;
  for (; t < nTiles; t += G, b ^= 1) {
    const int tn = t + G;
    if (tn < nTiles) pipe_issue<NS, MODE>(m, Xin, Xbase, tn, smem + (b ^ 1) * T::kBuf, hidNext);
    cp_async_commit();
    hidNext = halo_id(tn + G);
    cp_async_wait<1>();   // tile t's copies (all groups but the one just issued) have landed
    __syncthreads();
    unsigned char* B = smem + b * T::kBuf;
    const float4* bSL = reinterpret_cast<const float4*>(B + T::kSL);
    const float4* bX = reinterpret_cast<const float4*>(B + T::kX);
    const float4* bCP = reinterpret_cast<const float4*>(B + T::kCP);
    const float4* bCS = reinterpret_cast<const float4*>(B + T::kCS);
    const float2* bQ = reinterpret_cast<const float2*>(B + T::kQ);
    const float4* bHX = reinterpret_cast<const float4*>(B + T::kHX);
    const float4* bHP = reinterpret_cast<const float4*>(B + T::kHP);
    const float4* bXB = reinterpret_cast<const float4*>(B + T::kXB);
    const float2* bQB = reinterpret_cast<const float2*>(B + T::kQB);
    const int base = t * kBlock, c = base + tid;
    float hOut = 0.0f;
    bool wetOut = false;
    const int mem = (!FUSED && s.nMembers > 0 && c < n) ? member_of(s, c) : -1;   // an ensemble member's own step
    if (c < n) {
      float4 sl[NS];
#pragma unroll
      for (int k = 0; k < NS; ++k) sl[k] = bSL[k * kBlock + tid];
      stage_cell<NS, MODE, true, RS>(m, s, Xin.x, bX, bCP, bHX, bHP, base, c, sl, bX[tid], bCP[tid], bCS[tid], bQ, bXB,
                                 bQB, tid, mem >= 0 ? s.dtMf[mem] : dtShared, FUSED ? f.totalIn : m.totalA, Xout,
                                 nullptr, cfl, cand, hOut, wetOut);
    }
    if (!FUSED && cfl && s.nMembers > 0) {   // members: each tile's candidates into their members' minima
      member_min_publish_f(s, cand, mem);
      cand = INFINITY;
    }
    if (FUSED && m.nInlet > 0) fused_inlet_totals<NS>(m, f, c, hOut, wetOut);
    __syncthreads();   // buffer b is refilled at the top of the next iteration
  }
  cp_async_wait<0>();
  if (FUSED && f.record && blockIdx.x == 0 && tid == 0) fused_record(s, f);
  if (cfl && (FUSED || s.nMembers == 0)) block_min_publish_f(cand, FUSED ? s.cflMinF + (1 - f.parity) : s.cflMinF);
}

// ---------------------------------------------------------------------------
// Face-once fused stage (meshes of degree <= 4)
// ---------------------------------------------------------------------------
// The gather kernels evaluate every interior face twice, once from each side,
// as the reference's per-cell loop does (semi_discretize_swe_2D.jl:286-419),
// and the face arithmetic is most of their instructions.  Here one block takes
// one 256-cell tile in three phases:
//  1. loads and side records: every global load of the tile is issued first --
//     the own cells' records, the tile's face list (DevMesh::FL) and the inputs
//     of phase 3 by asynchronous copies into shared memory, the halo (the
//     tile's out-of-tile neighbours, DevMesh::halo) as soon as its ids arrive;
//     each own and halo cell is clamped once and its side record formed
//     (xi and hstill pairs, clamped depth, masked momenta, velocity, sqrt(h));
//  2. faces: one thread per face-list entry: a wet-wet face is evaluated once
//     and gives both cells' terms (roe_face_wet_f32); a face with a dry side
//     is evaluated from each of its in-tile sides, as the per-cell loop does;
//     a boundary face from its cell; the terms times the face length go to
//     shared memory;
//  3. cells: each cell adds its slots' terms in slot order (deterministic, no
//     atomics) and finishes the stage as the gather kernels do (stage_finish).
// A face between two tiles is listed in both, oriented from its lower cell id,
// so both tiles form the same flux bits and the continuity terms of every
// wet-wet face cancel exactly.
constexpr int kFaceRec = kBlock + kHaloMax;   // side records per tile: own cells, then halo cells

// Shared-memory layout of k_stage_face_f32, in 16-byte units: side records
// R0 {xi_hi, xi_lo, hstill_hi, hstill_lo}, R1 {h, hu, hv, excess}, R2 {u, v,
// sqrt h, dry ? 1 : 0}, R3 {zb, n} (8 bytes each); two terms per face; the
// face list; the own cells' CS and lo parts and, in stage 2, the base state.
struct FaceSmem {
  static constexpr int kR0 = 0, kR1 = kFaceRec, kR2 = 2 * kFaceRec, kR3 = 3 * kFaceRec;
  static constexpr int kC = kR3 + kFaceRec / 2;
  __host__ __device__ static int fl(int faceMax) { return kC + 2 * faceMax; }
  __host__ __device__ static int cs(int faceMax) { return fl(faceMax) + faceMax; }
  __host__ __device__ static int q(int faceMax) { return cs(faceMax) + kBlock; }
  __host__ __device__ static int xb(int faceMax) { return q(faceMax) + kBlock / 2; }
  __host__ __device__ static int qb(int faceMax) { return xb(faceMax) + kBlock; }
  __host__ __device__ static uint32_t bytes(int faceMax, int mode) {
    return (uint32_t)(mode == kModeStage2 ? qb(faceMax) + kBlock / 2 : xb(faceMax)) * 16u;
  }
};

__device__ __forceinline__ void face_side_record(const DevMesh& m, float4* R0, float4* R1, float4* R2, float2* R3,
                                                 int i, float4 x, float4 p) {
  const SideF32 d = make_side_f32(x, p, m.hsmf, m.hsmLo);
  const OwnF32 o = own_f32(d.s, m.gf);
  R0[i] = make_float4(x.x, x.y, p.x, p.y);
  R1[i] = make_float4(d.s.h, d.s.hu, d.s.hv, d.excess);
  R2[i] = make_float4(o.u, o.v, o.s, d.s.dry ? 1.0f : 0.0f);
  R3[i] = make_float2(p.z, p.w);
}

__device__ __forceinline__ Side<float> face_side(float4 r0, float4 r1, float4 r2, float zb) {
  Side<float> s;
  s.xi = r0.x;
  s.hst = r0.z;
  s.h = r1.x;
  s.hu = r1.y;
  s.hv = r1.z;
  s.zb = zb;
  s.dry = r2.w != 0.0f;
  return s;
}

// Pre-balanced pressure g/2 (smooth_pow2(xi) + 2 xi hstill) of a side (own_f32's p).
__device__ __forceinline__ float face_pressure(const DevMesh& m, float xi, float hst) {
  return 0.5f * m.gf * (smooth_pow2(xi) + 2.0f * xi * hst);
}

// Terms of face entry i (record rec) into C[2 i] (side a) and C[2 i + 1] (side b).
// base: the tile's first cell; haloIds: the tile's halo cell ids (DevMesh::halo).
template <int RS>
__device__ __forceinline__ void face_terms(const DevMesh& m, const float4* R0, const float4* R1, const float4* R2,
                                           const float2* R3, float4* C, int i, float4 rec,
                                           const double* __restrict__ totalA, int32_t* flags, int base,
                                           const int32_t* __restrict__ haloIds) {
  const int32_t w = __float_as_int(rec.w);
  const float nx = rec.x, ny = rec.y, len = rec.z;
  const int rs = RS >= 0 ? RS : m.riemann;
  float F[3];
  const int a = w & 1023;
  const float4 a0 = R0[a], a1 = R1[a], a2 = R2[a];
  if (w >= 0) {
    const int b = (w >> 10) & 1023;
    const bool aOwn = (w >> 20) & 1, bOwn = (w >> 21) & 1;
    const float4 b0 = R0[b], b1 = R1[b], b2 = R2[b];
    const float dxi = (b0.x - a0.x) + (b0.y - a0.y);    // xi_b - xi_a from the pairs
    const float dhst = (b0.z - a0.z) + (b0.w - a0.w);   // hstill_b - hstill_a
    if (a2.w == 0.0f && b2.w == 0.0f) {                 // wet-wet: once for both cells
      const FaceSideF32 A{a0.x, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
      const FaceSideF32 B{b0.x, b0.z, b1.x, b1.y, b1.z, b2.x, b2.y, b2.z};
      const float dp = rs == kRiemannHll ? hll_face_wet_f32(A, B, dxi, dhst, m.gf, nx, ny, F)
                                         : roe_face_wet_f32(A, B, dxi, dhst, m.gf, nx, ny, F);
      const float c0 = F[0] * len;
      const float2 c12 = mul2(p2(F[1], F[2]), p2(len));
      if (aOwn) C[2 * i] = make_float4(c0, c12.x, c12.y, 0.0f);
      if (bOwn) {   // -c_a + dp n L
        const float2 b12 = fma2(p2(dp * len), p2(nx, ny), p2(-c12.x, -c12.y));
        C[2 * i + 1] = make_float4(-c0, b12.x, b12.y, 0.0f);
      }
    } else {                                            // a dry side: each in-tile side from its own cell
      const Side<float> sa = face_side(a0, a1, a2, R3[a].x), sb = face_side(b0, b1, b2, R3[b].x);
      int bank = -1;   // the wall test in FP64 (bank_wall_f64); the same from either side
      if (sa.dry != sb.dry) {
        const int ga = a < kBlock ? base + a : __ldg(&haloIds[a - kBlock]);
        const int gb = b < kBlock ? base + b : __ldg(&haloIds[b - kBlock]);
        bank = sa.dry ? bank_wall_f64(m, b0.x, b0.y, gb, ga) : bank_wall_f64(m, a0.x, a0.y, ga, gb);
      }
      if (aOwn) {
        const float pa = face_pressure(m, a0.x, a0.z);
        riemann_flux<float>(rs, sa, sb, dxi, m.gf, nx, ny, m.hsmf, F, bank);
        C[2 * i] = make_float4(F[0] * len, (F[1] - pa * nx) * len, (F[2] - pa * ny) * len, 0.0f);
      }
      if (bOwn) {
        const float pb = face_pressure(m, b0.x, b0.z);
        riemann_flux<float>(rs, sb, sa, -dxi, m.gf, -nx, -ny, m.hsmf, F, bank);
        C[2 * i + 1] = make_float4(F[0] * len, (F[1] + pb * nx) * len, (F[2] + pb * ny) * len, 0.0f);
      }
    }
    return;
  }
  // boundary face of own cell a: its ghost state (bc_2D.jl:640-834)
  const int32_t bf = (w >> 10) & 0x1FFFFF;
  const float2 a3 = R3[a];
  const Side<float> L = face_side(a0, a1, a2, a3.x);
  const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
  if (type == kBcInletQ && !(totalA[grp] > 1e-10)) atomicOr(flags, 2);   // bc_2D.jl:679
  const Side<float> R = ghost_state<float>(L, type, nx, ny, m.hsmf, type == kBcExitH ? (float)m.exitWse[grp] : 0.0f,
                                           type == kBcInletQ ? (float)m.inletQ[grp] : 0.0f,
                                           type == kBcInletQ ? (float)totalA[grp] : 1.0f, m.bfLp23f[bf], a3.y);
  float dxi = (R.h - L.h) + a1.w;
  if (type == kBcExitH && !R.dry) dxi = m.bfExitRel[bf] - (a0.x + a0.y);
  int bank = -1;
  if (type == kBcExitH && L.dry != R.dry)
    bank = L.dry ? bank_exit_f64(m, grp, base + a) : bank_wall_f64(m, a0.x, a0.y, base + a, base + a);
  const float pa = face_pressure(m, a0.x, a0.z);
  if (!L.dry && !R.dry) {
    OwnF32 o;
    o.u = a2.x; o.v = a2.y; o.s = a2.z; o.p = pa;
    o.fxx = L.hu * o.u; o.fxy = L.hu * o.v; o.fyx = L.hv * o.u; o.fyy = L.hv * o.v;
    if (rs == kRiemannHll) hll_flux_wet_f32(L, o, R, dxi, 0.0f, m.gf, nx, ny, F);
    else roe_flux_wet_f32(L, o, R, dxi, 0.0f, m.gf, nx, ny, F);
  } else {
    riemann_flux<float>(rs, L, R, dxi, m.gf, nx, ny, m.hsmf, F, bank);
    F[1] -= pa * nx;
    F[2] -= pa * ny;
  }
  C[2 * i] = make_float4(F[0] * len, F[1] * len, F[2] * len, 0.0f);
}

template <int NS, int MODE, bool FUSED, int RS, int MINB = 4>
__global__ void __launch_bounds__(kBlock, MINB)
    k_stage_face_f32(DevMesh m, DevScalars s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl, StageFuse f) {
  pdl_enter();
  extern __shared__ float4 fsm[];
  using L = FaceSmem;
  float4* R0 = fsm + L::kR0;
  float4* R1 = fsm + L::kR1;
  float4* R2 = fsm + L::kR2;
  float2* R3 = reinterpret_cast<float2*>(fsm + L::kR3);
  float4* C = fsm + L::kC;
  float4* sFL = fsm + L::fl(m.faceMax);
  float4* sCS = fsm + L::cs(m.faceMax);
  float2* sQ = reinterpret_cast<float2*>(fsm + L::q(m.faceMax));
  float4* sXB = fsm + L::xb(m.faceMax);
  float2* sQB = reinterpret_cast<float2*>(fsm + L::qb(m.faceMax));
  __shared__ float dtShared;
  const int tile = blockIdx.x, tid = threadIdx.x;
  const int base = tile * kBlock, c = base + tid;
  const bool active = c < m.n;
  const double* totalIn = FUSED ? f.totalIn : m.totalA;
  // phase 1: every load of the tile, then the side records
  const int hid = tid < kHaloMax ? __ldg(&m.halo[(size_t)tile * kHaloMax + tid]) : -1;
  const int f0 = __ldg(&m.FLoff[tile]), nf = __ldg(&m.FLoff[tile + 1]) - f0;
  float4 xin, cp;
  uint2 refs;
  if (active) {
    xin = __ldg(&Xin.x[c]);
    cp = __ldg(&m.CP[c]);
    refs = __ldg(&m.FR[c]);
    cp_async16(&sCS[tid], &m.CS[c]);
    cp_async8(&sQ[tid], &Xin.q[c]);
    if constexpr (MODE == kModeStage2) {
      cp_async16(&sXB[tid], &Xbase.x[c]);
      cp_async8(&sQB[tid], &Xbase.q[c]);
    }
  }
  for (int i = tid; i < nf; i += kBlock) cp_async16(&sFL[i], &m.FL[f0 + i]);
  cp_async_commit();
  float4 xh, ph;
  if (hid >= 0) {
    xh = __ldg(&Xin.x[hid]);
    ph = __ldg(&m.CP[hid]);
  }
  if (active) face_side_record(m, R0, R1, R2, R3, tid, xin, cp);
  if (hid >= 0) face_side_record(m, R0, R1, R2, R3, kBlock + tid, xh, ph);
  if (tid == 0) dtShared = FUSED ? (float)fused_dt(s, f) : *s.dtf;
  cp_async_wait<0>();
  __syncthreads();
  // phase 2: the tile's faces
  for (int i = tid; i < nf; i += kBlock)
    face_terms<RS>(m, R0, R1, R2, R3, C, i, sFL[i], totalIn, s.flags, base, m.halo + (size_t)tile * kHaloMax);
  __syncthreads();
  // phase 3: each cell's terms in slot order, then the stage update
  float cand = INFINITY, hOut = 0.0f;
  bool wetOut = false;
  if (active) {
    float4 sl[NS];
    float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const unsigned int ref = ((k < 2 ? refs.x : refs.y) >> (16 * (k & 1))) & 0xFFFFu;
      sl[k] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(kNoFace));
      if (ref == 0xFFFFu) continue;
      const float4 t = C[ref];
      g0 += t.x;
      const float2 g12 = add2(p2(g1, g2), p2(t.y, t.z));
      g1 = g12.x;
      g2 = g12.y;
      if (cfl) {   // the slot's geometry for the CFL candidate (|u.n| does not depend on the side)
        const float4 g = sFL[ref >> 1];
        sl[k] = make_float4(g.x, g.y, g.z, 0.0f);
      }
    }
    const float4 r1 = R1[tid], r2 = R2[tid];
    SideF32 Ls;
    Ls.s = face_side(R0[tid], r1, r2, cp.z);
    Ls.xlo = xin.y;
    Ls.excess = r1.w;
    const float dt = MODE == kModeRhs ? 0.0f : dtShared;
    stage_finish<NS, MODE>(m, s, Ls, g0, g1, g2, c, sl, xin, cp, sCS[tid], sQ, sXB, sQB, tid, dt, Xout, nullptr,
                           cfl, cand, hOut, wetOut);
  }
  if (FUSED && f.record && blockIdx.x == 0 && tid == 0) fused_record(s, f);
  if (cfl) block_min_publish_f(cand, FUSED ? s.cflMinF + (1 - f.parity) : s.cflMinF);
  if (FUSED && m.nInlet > 0) fused_inlet_totals<NS>(m, f, c, hOut, wetOut);
}

template <int NS>
__global__ void __launch_bounds__(kBlock) k_cfl_f32(DevMesh m, DevScalars s, StateF32 X) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  float cand = INFINITY;
  if (c < m.n) {
    const float4 x = X.x[c];
    float4 sl[NS];
    load_slots<NS>(m, c, sl);
    const SideF32 L = make_side_f32(x, m.CP[c], m.hsmf, m.hsmLo);
    cand = cfl_candidate_f32<NS>(m, sl, L.s.h, x.z, x.w, L.s.dry, m.CS[c].z);
  }
  if (s.nMembers > 0) member_min_publish_f(s, cand, c < m.n ? member_of(s, c) : -1);
  else block_min_publish_f(cand, s.cflMinF);
}

// Group g = blockIdx.y, its faces [o0 + p kBlock, o0 + (p + 1) kBlock) in
// block p = blockIdx.x, one a thread (a group's faces over m.inletParts blocks
// instead of one, whose threads each took several faces one after another);
// the last block of the group to finish adds the blocks' sums in block order
// (deterministic).
__global__ void __launch_bounds__(kBlock) k_inlet_total_f32(DevMesh m, DevScalars s, StateF32 X) {
  const int g = blockIdx.y, p = blockIdx.x, P = gridDim.x;
  const int o0 = m.inletOff[g], o1 = m.inletOff[g + 1];
  const int i = o0 + p * kBlock + threadIdx.x;
  double v = 0.0;
  if (i < o1) {
    const int c = m.inletCell[i];
    const float4 cp = m.CP[c];
    const SideF32 L = make_side_f32(X.x[c], cp, m.hsmf, m.hsmLo);
    v = L.s.dry ? 0.0 : m.inletLp53[i] * (double)L.s.h / (double)cp.w;
  }
  const double b = block_sum(v);
  __shared__ int isLast;
  if (threadIdx.x == 0) {
    m.inletPart[(size_t)g * P + p] = b;
    __threadfence();
    isLast = atomicAdd(&m.inletTicket[g], 1u) == (unsigned int)P - 1u;
  }
  __syncthreads();
  if (!isLast || threadIdx.x != 0) return;
  __threadfence();
  double t = 0.0;
  for (int q = 0; q < P; ++q) t += __ldcg(&m.inletPart[(size_t)g * P + q]);
  m.totalA[g] = t;
  if (!(t > 1e-10)) atomicOr(s.flags, 2);
  m.inletTicket[g] = 0u;
}

// ---------------------------------------------------------------------------
// Bookkeeping and renumbering
// ---------------------------------------------------------------------------
__global__ void k_step_begin(DevScalars s, int cflMode, double cfl) {
  if (s.nMembers > 0) {   // an ensemble: each member's own step (one block)
    const int k = *s.stepIdx;
    for (int mm = threadIdx.x; mm < s.nMembers; mm += blockDim.x) {
      double dt = *s.dt;
      if (cflMode) {
        dt = cfl * fmin(__longlong_as_double((long long)s.cflMinM[mm]), (double)__uint_as_float(s.cflMinMF[mm]));
        if (!(dt >= s.dtMin)) atomicOr(s.flags, 8);   // the member's step collapsed (or is NaN)
        s.cflMinM[mm] = (unsigned long long)__double_as_longlong(INFINITY);
        s.cflMinMF[mm] = __float_as_uint(INFINITY);
      }
      s.dtM[mm] = dt;
      s.dtMf[mm] = (float)dt;
      if (k < s.dtCap) s.dtHistM[(size_t)k * s.nMembers + mm] = dt;
      s.tM[mm] += dt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {   // the context's own record: member 0's step
      if (cflMode) *s.dt = s.dtM[0];
      *s.dtf = (float)*s.dt;
      if (k < s.dtCap) s.dtHist[k] = *s.dt;
      *s.stepIdx = k + 1;
      *s.tSum += *s.dt;
    }
    return;
  }
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (cflMode) {
    const double m = fmin(__longlong_as_double((long long)*s.cflMin), (double)__uint_as_float(*s.cflMinF));
    *s.dt = cfl * m;
    if (!(*s.dt >= s.dtMin)) atomicOr(s.flags, 8);   // the step collapsed (or is NaN)
    *s.cflMin = (unsigned long long)__double_as_longlong(INFINITY);
    *s.cflMinF = __float_as_uint(INFINITY);
  }
  *s.dtf = (float)*s.dt;
  const int k = *s.stepIdx;
  if (k < s.dtCap) s.dtHist[k] = *s.dt;
  *s.stepIdx = k + 1;
  *s.tSum += *s.dt;
}

__global__ void k_reset_cfl(DevScalars s, int p) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  s.cflMin[p] = (unsigned long long)__double_as_longlong(INFINITY);
  s.cflMinF[p] = __float_as_uint(INFINITY);
}

__global__ void k_reset_scalars(DevScalars s) {
  for (int mm = threadIdx.x; mm < s.nMembers; mm += blockDim.x) {
    s.cflMinM[mm] = (unsigned long long)__double_as_longlong(INFINITY);
    s.cflMinMF[mm] = __float_as_uint(INFINITY);
    s.tM[mm] = 0.0;
  }
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  s.cflMin[0] = s.cflMin[1] = (unsigned long long)__double_as_longlong(INFINITY);
  s.cflMinF[0] = s.cflMinF[1] = __float_as_uint(INFINITY);
  *s.stepIdx = 0;
  *s.tSum = 0.0;
  *s.flags = 0;
}

__global__ void k_gather_f64(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ user,
                             double* __restrict__ dev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  dev[i] = user[o];
  dev[n + i] = user[n + o];
  dev[2 * n + i] = user[2 * n + o];
}

__global__ void k_scatter_f64(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ dev,
                              double* __restrict__ user) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  user[o] = dev[i];
  user[n + o] = dev[n + i];
  user[2 * n + o] = dev[2 * n + i];
}

// One device-order field to the caller's order: user[perm[i]] = dev[i] (+ add[i]).
__global__ void k_scatter_field_f64(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ dev,
                                    const double* __restrict__ add, double* __restrict__ user) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  user[perm[i]] = add ? dev[i] + add[i] : dev[i];
}

__device__ __forceinline__ void split(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

__global__ void k_gather_f32(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ user, StateF32 X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  float xh, xl, uh, ul, vh, vl;
  split(user[o], xh, xl);
  split(user[n + o], uh, ul);
  split(user[2 * n + o], vh, vl);
  X.x[i] = make_float4(xh, xl, uh, vh);
  X.q[i] = make_float2(ul, vl);
}

__global__ void k_scatter_f32(int32_t n, const int32_t* __restrict__ perm, StateF32 X, double* __restrict__ user) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  const float4 x = X.x[i];
  const float2 q = X.q[i];
  user[o] = (double)x.x + (double)x.y;
  user[n + o] = (double)x.z + (double)q.x;
  user[2 * n + o] = (double)x.w + (double)q.y;
}

__global__ void k_flush(uint4* buf, size_t n16) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4((unsigned)i, 1u, 2u, 3u);
}

// Reads n16 16-byte words; the store is taken only if the words XOR to a
// value the flush never writes, which keeps the loads alive.
__global__ void k_flush_read(uint4* buf, size_t n16) {
  unsigned int acc = 0u;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = __ldcg(&buf[i]);
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0xFFFFFFFFu) buf[0].x = acc;
}

}  // namespace

void launch_inlet_total_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st) {
  launch_resistance_f32(m, X, st);
  if (m.nInlet > 0) k_inlet_total_f32<<<dim3(m.inletParts, m.nInlet), kBlock, 0, st>>>(m, s, X);
}
namespace {
// The fused gather kernel's shapes (DevMesh::stageVariant, the autotuner's
// candidates; the same arithmetic in each): 0 the default, 256-cell blocks
// with the register budget of 4 resident per SM (64 registers); 1 the same
// blocks at 3 per SM (80 registers); 2 512-cell blocks at 2 per SM and 3
// 128-cell blocks at 8 per SM (64 registers, as 0).
template <int NS, int MODE, int RS>
void launch_gather_shape(int v, const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                         double* Rout, int cfl, const StageFuse& f, cudaStream_t st) {
  auto grid = [&](int tb) { return (m.n + tb - 1) / tb; };
  if (v == 1)
    launch_k(true, k_stage_f32<NS, true, MODE, RS, 3>, grid(kBlock), kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  else if (v == 2)
    launch_k(true, k_stage_f32<NS, true, MODE, RS, 2, 512>, grid(512), 512, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  else if (v == 3)
    launch_k(true, k_stage_f32<NS, true, MODE, RS, 8, 128>, grid(128), 128, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  else
    launch_k(true, k_stage_f32<NS, true, MODE, RS>, grid(kBlock), kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
}

template <int NS, bool FUSED>
void launch_stage_ns(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                     double* Rout, int cfl, const StageFuse& f, cudaStream_t st) {
  const int nb = blocks_for(m.n);
  if constexpr (FUSED) {   // the fused stages: the solver fixed per instance, the shape by variant
    const bool hll = m.riemann == kRiemannHll;
    const int v = NS <= 4 ? m.stageVariant : 0;
    if (mode == kModeStage1) {
      if (hll) launch_gather_shape<NS, kModeStage1, kRiemannHll>(v, m, s, Xin, Xbase, Xout, Rout, cfl, f, st);
      else launch_gather_shape<NS, kModeStage1, kRiemannRoe>(v, m, s, Xin, Xbase, Xout, Rout, cfl, f, st);
    } else if (mode == kModeStage2) {
      if (hll) launch_gather_shape<NS, kModeStage2, kRiemannHll>(v, m, s, Xin, Xbase, Xout, Rout, cfl, f, st);
      else launch_gather_shape<NS, kModeStage2, kRiemannRoe>(v, m, s, Xin, Xbase, Xout, Rout, cfl, f, st);
    }
  } else if (mode == kModeStage1) {
    launch_k(true, k_stage_f32<NS, false, kModeStage1>, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  } else if (mode == kModeStage2) {
    launch_k(true, k_stage_f32<NS, false, kModeStage2>, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  } else {
    if (mode == kModeRhs)
      launch_k(true, k_stage_f32<NS, false, kModeRhs>, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
    else if (mode == kModeRhsF32)
      launch_k(true, k_stage_f32<NS, false, kModeRhsF32>, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
    else
      launch_k(true, k_stage_f32<NS, false, kModeEulerRef>, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, Rout, cfl, f);
  }
}
}  // namespace

namespace {
// Kernel of the fused stages: HG_STAGE_KERNEL = gather / pipe / tma forces
// one; otherwise DevMesh::stageKernel (hg_autotune's choice).  Measured on the
// 1M-cell reach (CUDA events, L2 flushed): gather 37.1 us, pipe 37.1 us per
// stage-1 launch, pipe 3 % faster per step; tma 41 us (its out-of-tile gathers
// inside the face loop leave barrier stalls at every tile).
int forced_stage_kernel() {
  static const int k = [] {
    const char* e = std::getenv("HG_STAGE_KERNEL");
    if (!e) return -1;
    if (std::strcmp(e, "gather") == 0) return (int)kStageGather;
    if (std::strcmp(e, "pipe") == 0) return (int)kStagePipe;
    if (std::strcmp(e, "tma") == 0) return (int)kStageTma;
    if (std::strcmp(e, "face") == 0) return (int)kStageFace;
    return -1;
  }();
  return k;
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// CTAs of a persistent kernel resident per SM (its grid: every CTA resident,
// so the tiles split evenly).
template <class Kernel>
int resident_ctas(Kernel k, uint32_t smem) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBlock, smem) != cudaSuccess || n < 1) n = 1;
  return n;
}

template <int NS, int MODE, int RS>
void launch_tma_rs(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                   const StageFuse& fu, cudaStream_t st) {
  using T = TmaTile<NS, MODE>;
  static const bool attr = [] {   // more than 48 KB of dynamic shared memory: opt in once
    cudaFuncSetAttribute(k_stage_tma_f32<NS, MODE, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::kSmem);
    return true;
  }();
  (void)attr;
  static const int grid = sm_count() * kTmaCtasPerSm;
  const int tiles = blocks_for(m.n);
  launch_k(true, k_stage_tma_f32<NS, MODE, RS>, tiles < grid ? tiles : grid, kBlock, T::kSmem, st, m, s, Xin, Xbase,
           Xout, cfl, fu);
}
template <int NS, int MODE>
void launch_tma(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                const StageFuse& fu, cudaStream_t st) {
  if (m.riemann == kRiemannHll) launch_tma_rs<NS, MODE, kRiemannHll>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_tma_rs<NS, MODE, kRiemannRoe>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}

template <int NS, int MODE, bool FUSED, int RS>
void launch_pipe_rs(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                    const StageFuse& fu, cudaStream_t st) {
  using T = PipeTile<NS, MODE>;
  static const bool attr = [] {   // more than 48 KB of dynamic shared memory: opt in once
    cudaFuncSetAttribute(k_stage_pipe_f32<NS, MODE, FUSED, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)T::kSmem);
    return true;
  }();
  (void)attr;
  static const int grid = sm_count() * resident_ctas(k_stage_pipe_f32<NS, MODE, FUSED, RS>, T::kSmem);
  const int tiles = blocks_for(m.n);
  launch_k(true, k_stage_pipe_f32<NS, MODE, FUSED, RS>, tiles < grid ? tiles : grid, kBlock, T::kSmem, st, m, s, Xin,
           Xbase, Xout, cfl, fu);
}
template <int NS, int MODE, bool FUSED>
void launch_pipe(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                 const StageFuse& fu, cudaStream_t st) {
  if (m.riemann == kRiemannHll) launch_pipe_rs<NS, MODE, FUSED, kRiemannHll>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_pipe_rs<NS, MODE, FUSED, kRiemannRoe>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}


template <int NS, int MODE, bool FUSED, int RS, int MINB>
void launch_face_minb(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                      const StageFuse& fu, cudaStream_t st) {
  static const bool attr = [] {   // more than 48 KB of dynamic shared memory: opt in once, for the largest tables
    cudaFuncSetAttribute(k_stage_face_f32<NS, MODE, FUSED, RS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)FaceSmem::bytes(kFaceMaxPerTile, MODE));
    return true;
  }();
  (void)attr;
  launch_k(true, k_stage_face_f32<NS, MODE, FUSED, RS, MINB>, blocks_for(m.n), kBlock,
           FaceSmem::bytes(m.faceMax, MODE), st, m, s, Xin, Xbase, Xout, cfl, fu);
}
// The register budget by variant: 4 blocks per SM (64 registers), or 3 (80).
template <int NS, int MODE, bool FUSED, int RS>
void launch_face_rs(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                    const StageFuse& fu, cudaStream_t st) {
  if (m.stageVariant == 1) launch_face_minb<NS, MODE, FUSED, RS, 3>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_face_minb<NS, MODE, FUSED, RS, 4>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}
template <int NS, int MODE, bool FUSED>
void launch_face(const DevMesh& m, const DevScalars& s, StateF32 Xin, StateF32 Xbase, StateF32 Xout, int cfl,
                 const StageFuse& fu, cudaStream_t st) {
  if (m.riemann == kRiemannHll) launch_face_rs<NS, MODE, FUSED, kRiemannHll>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_face_rs<NS, MODE, FUSED, kRiemannRoe>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}
template <int NS, bool FUSED = true>
void launch_face_mode(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                      int cfl, const StageFuse& fu, cudaStream_t st) {
  if (mode == kModeStage1) launch_face<NS, kModeStage1, FUSED>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_face<NS, kModeStage2, FUSED>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}

template <int NS, bool FUSED = true>
void launch_pipe_mode(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                      int cfl, const StageFuse& fu, cudaStream_t st) {
  if (mode == kModeStage1) launch_pipe<NS, kModeStage1, FUSED>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_pipe<NS, kModeStage2, FUSED>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}

template <int NS>
void launch_tma_mode(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                     int cfl, const StageFuse& fu, cudaStream_t st) {
  if (mode == kModeStage1) launch_tma<NS, kModeStage1>(m, s, Xin, Xbase, Xout, cfl, fu, st);
  else launch_tma<NS, kModeStage2>(m, s, Xin, Xbase, Xout, cfl, fu, st);
}
}  // namespace

int stage_kernel_forced() { return forced_stage_kernel(); }
int stage_variant_forced() {
  static const int v = [] {
    const char* e = std::getenv("HG_STAGE_VARIANT");
    return (e && e[0] >= '0' && e[0] <= '3' && e[1] == 0) ? e[0] - '0' : -1;
  }();
  return v;
}

bool stage_kernel_usable(const DevMesh& m, int k, int mode, StateF32 Xin, StateF32 Xbase) {
  auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  auto a8 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; };
  if (k == kStageGather) return true;
  if (m.nslot > 4) return false;
  if (k == kStageFace)   // cp.async: 16-byte records 16-byte aligned, the lo parts 8-byte aligned
    return m.FL && m.FLoff && m.FR && m.halo && m.faceMax <= kFaceMaxPerTile && a16(m.CS) && a16(m.FL) &&
           a8(Xin.q) && (mode != kModeStage2 || (a16(Xbase.x) && a8(Xbase.q)));
  if (k == kStagePipe)   // cp.async: 16-byte records 16-byte aligned, the lo parts 8-byte aligned
    return m.SLp && m.halo && a16(m.SLp) && a16(m.CP) && a16(m.CS) && a16(Xin.x) && a8(Xin.q) &&
           (mode != kModeStage2 || (a16(Xbase.x) && a8(Xbase.q)));
  // bulk copies: 16-byte aligned sources (tile offsets are multiples of 2048 B);
  // a state view whose lo parts start 8 bytes off takes another kernel
  return a16(m.SL) && a16(m.CP) && a16(m.CS) && a16(Xin.x) && a16(Xin.q) &&
         (mode != kModeStage2 || (a16(Xbase.x) && a16(Xbase.q)));
}

void launch_stage_f32(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                      double* Rout, bool cfl, cudaStream_t st) {
  const int f = cfl ? 1 : 0;
  const StageFuse nf{};
  // Stages of unfused steps (ensembles, state-dependent resistance) take the
  // persistent pipelined kernel wherever it can run, whatever the autotuner
  // chose for fused steps: its unfused instance and the gather kernel's differ
  // in the last FP32 bit of a few cells (the compiler contracts the same
  // source differently), so a fixed choice keeps runs reproducible.
  // HG_STAGE_KERNEL=gather (or tma) selects the gather kernel here.
  const int forced = stage_kernel_forced();
  if ((mode == kModeStage1 || mode == kModeStage2) && (forced < 0 || forced == kStagePipe) &&
      stage_kernel_usable(m, kStagePipe, mode, Xin, Xbase)) {
    if (m.nslot <= 3) launch_pipe_mode<3, false>(m, s, mode, Xin, Xbase, Xout, f, nf, st);
    else launch_pipe_mode<4, false>(m, s, mode, Xin, Xbase, Xout, f, nf, st);
    return;
  }
  if (m.nslot <= 3) launch_stage_ns<3, false>(m, s, mode, Xin, Xbase, Xout, Rout, f, nf, st);
  else if (m.nslot <= 4) launch_stage_ns<4, false>(m, s, mode, Xin, Xbase, Xout, Rout, f, nf, st);
  else launch_stage_ns<8, false>(m, s, mode, Xin, Xbase, Xout, Rout, f, nf, st);
}

namespace {
// Fused stages with Manning's n from a function of the state (RESFN): the
// gather kernel in its default shape.
template <int NS>
void launch_stage_resfn(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                        int cfl, const StageFuse& f, cudaStream_t st) {
  const bool hll = m.riemann == kRiemannHll;
  const int nb = blocks_for(m.n);
  double* none = nullptr;
  if (mode == kModeStage1) {
    auto k = hll ? k_stage_f32<NS, true, kModeStage1, kRiemannHll, 0, kBlock, true>
                 : k_stage_f32<NS, true, kModeStage1, kRiemannRoe, 0, kBlock, true>;
    launch_k(true, k, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, none, cfl, f);
  } else if (mode == kModeStage2) {
    auto k = hll ? k_stage_f32<NS, true, kModeStage2, kRiemannHll, 0, kBlock, true>
                 : k_stage_f32<NS, true, kModeStage2, kRiemannRoe, 0, kBlock, true>;
    launch_k(true, k, nb, kBlock, 0, st, m, s, Xin, Xbase, Xout, none, cfl, f);
  }
}
}  // namespace

void launch_stage_f32_fused(const DevMesh& m0, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase,
                            StateF32 Xout, const StageFuse& fu, cudaStream_t st) {
  const int f = (!fu.record && fu.cflMode) ? 1 : 0;   // stage 2 publishes the next CFL minimum
  if (m0.res.kind != kResConstant) {   // n(h, Umag, ks) of the state, in the kernel
    if (m0.nslot <= 3) launch_stage_resfn<3>(m0, s, mode, Xin, Xbase, Xout, f, fu, st);
    else if (m0.nslot <= 4) launch_stage_resfn<4>(m0, s, mode, Xin, Xbase, Xout, f, fu, st);
    else launch_stage_resfn<8>(m0, s, mode, Xin, Xbase, Xout, f, fu, st);
    return;
  }
  const int forced = forced_stage_kernel();
  DevMesh m = m0;
  if (stage_variant_forced() >= 0) m.stageVariant = stage_variant_forced();
  const int k = forced >= 0 ? forced : m.stageKernel;
  if (k == kStageFace && stage_kernel_usable(m, k, mode, Xin, Xbase)) {
    if (m.nslot <= 3) launch_face_mode<3>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    else launch_face_mode<4>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    return;
  }
  if (k == kStagePipe && stage_kernel_usable(m, k, mode, Xin, Xbase)) {
    if (m.nslot <= 3) launch_pipe_mode<3>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    else launch_pipe_mode<4>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    return;
  }
  if (k == kStageTma && stage_kernel_usable(m, k, mode, Xin, Xbase)) {
    if (m.nslot <= 3) launch_tma_mode<3>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    else launch_tma_mode<4>(m, s, mode, Xin, Xbase, Xout, f, fu, st);
    return;
  }
  if (m.nslot <= 3) launch_stage_ns<3, true>(m, s, mode, Xin, Xbase, Xout, nullptr, f, fu, st);
  else if (m.nslot <= 4) launch_stage_ns<4, true>(m, s, mode, Xin, Xbase, Xout, nullptr, f, fu, st);
  else launch_stage_ns<8, true>(m, s, mode, Xin, Xbase, Xout, nullptr, f, fu, st);
}
int stage_blocks_f32(const DevMesh& m) { return blocks_for(m.n); }
void launch_reset_cfl(const DevScalars& s, int parity, cudaStream_t st) { k_reset_cfl<<<1, 32, 0, st>>>(s, parity); }
void launch_cfl_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st) {
  if (m.nslot <= 3) k_cfl_f32<3><<<blocks_for(m.n), kBlock, 0, st>>>(m, s, X);
  else if (m.nslot <= 4) k_cfl_f32<4><<<blocks_for(m.n), kBlock, 0, st>>>(m, s, X);
  else k_cfl_f32<8><<<blocks_for(m.n), kBlock, 0, st>>>(m, s, X);
}
void launch_step_begin(const DevScalars& s, bool cflMode, double cfl, cudaStream_t st) {
  k_step_begin<<<1, s.nMembers > 0 ? 256 : 32, 0, st>>>(s, cflMode ? 1 : 0, cfl);
}
void launch_reset_scalars(const DevScalars& s, cudaStream_t st) { k_reset_scalars<<<1, 32, 0, st>>>(s); }
void launch_gather_state_f64(int32_t n, const int32_t* perm, const double* user, double* dev, cudaStream_t st) {
  k_gather_f64<<<blocks_for(n), kBlock, 0, st>>>(n, perm, user, dev);
}
void launch_scatter_state_f64(int32_t n, const int32_t* perm, const double* dev, double* user, cudaStream_t st) {
  k_scatter_f64<<<blocks_for(n), kBlock, 0, st>>>(n, perm, dev, user);
}
void launch_scatter_field_f64(int32_t n, const int32_t* perm, const double* dev, const double* add, double* user,
                              cudaStream_t st) {
  k_scatter_field_f64<<<blocks_for(n), kBlock, 0, st>>>(n, perm, dev, add, user);
}
void launch_gather_state_f32(int32_t n, const int32_t* perm, const double* user, StateF32 dev, cudaStream_t st) {
  k_gather_f32<<<blocks_for(n), kBlock, 0, st>>>(n, perm, user, dev);
}
void launch_scatter_state_f32(int32_t n, const int32_t* perm, StateF32 dev, double* user, cudaStream_t st) {
  k_scatter_f32<<<blocks_for(n), kBlock, 0, st>>>(n, perm, dev, user);
}
int launch_flush(void* buf, size_t bytes, cudaStream_t st) {
  // write the first half, then read the second: the L2 is left holding clean
  // lines of the flush buffer only (no state data, nothing to write back)
  const size_t half16 = bytes / 32;
  k_flush<<<152 * 8, 256, 0, st>>>(static_cast<uint4*>(buf), half16);
  k_flush_read<<<152 * 8, 256, 0, st>>>(static_cast<uint4*>(buf) + half16, half16);
  return 2;
}

}  // namespace hg
