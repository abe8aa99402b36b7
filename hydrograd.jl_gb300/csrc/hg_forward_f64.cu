// FP64 stage kernels (the parity path).
//
// Compiled with --fmad=false: every product and sum is rounded on its own, as
// in the reference (Julia does not contract a*b+c) and in the oracle, so the
// wet/dry decisions h <= h_small, taken on sums near the threshold, come out
// the same.  Each thread owns one cell (device order) and gathers its faces in
// the reference's local order (compute_inviscid_fluxes,
// src/fvm/discretization/semi_discretize_swe_2D.jl:286-419): clamp, ghost
// state, Roe flux, -sum F L / A, Manning friction + bed-slope source, then the
// stage update and the depth-positivity clamp.  Gather form: no atomics, and
// the per-cell summation order is the reference's.
#include <cfloat>
#include <cmath>

#include "hg_device.cuh"
#include "hg_members.cuh"
#include "hg_reduce.cuh"
#include "hg_state.hpp"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = 256;

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

// ---------------------------------------------------------------------------
// FP64 path
// ---------------------------------------------------------------------------
__device__ __forceinline__ Side<double> load_f64(const DevMesh& m, const double* __restrict__ Q, int j) {
  Side<double> s;
  s.xi = Q[j];
  s.hst = m.hst[j];
  s.zb = m.zb[j];
  double h = s.xi + s.hst;          // h = xi + hstill, clamped (semi_discretize_swe_2D.jl:101-106)
  s.dry = h <= m.hsm;
  s.h = s.dry ? m.hsm : h;
  s.hu = s.dry ? 0.0 : Q[m.n + j];
  s.hv = s.dry ? 0.0 : Q[2 * m.n + j];
  return s;
}

// The quantities of a wet own cell that the reference's Roe solver forms on
// every one of its faces (swe_2D_solvers.jl:79-127), formed once: the same
// operations in the same order, so the fluxes are bit-identical.
struct OwnF64 {
  double uL, vL, sL, pL;
  double hu_uL_pL, hu_vL, hv_uL, hv_vL_pL;   // L.hu*uL + pL, L.hu*vL, L.hv*uL, L.hv*vL + pL
};

__device__ __forceinline__ OwnF64 own_f64(const Side<double>& L, double g) {
  OwnF64 o;
  o.uL = L.hu / L.h;
  o.vL = L.hv / L.h;
  o.sL = smooth_sqrt(L.h);
  o.pL = 0.5 * g * (smooth_pow2(L.xi) + 2.0 * L.xi * L.hst);
  o.hu_uL_pL = L.hu * o.uL + o.pL;
  o.hu_vL = L.hu * o.vL;
  o.hv_uL = L.hv * o.uL;
  o.hv_vL_pL = L.hv * o.vL + o.pL;
  return o;
}

// roe_flux<double> of a face with both sides wet (the branch-free path), with
// the own cell's terms from own_f64.
__device__ __forceinline__ void roe_flux_wet_f64(const Side<double>& L, const OwnF64& o, const Side<double>& R,
                                                 double dxi, double g, double nx, double ny, double F[3]) {
  const double uL = o.uL, vL = o.vL, uR = R.hu / R.h, vR = R.hv / R.h;
  const double sL = o.sL, sR = smooth_sqrt(R.h);
  const double hRoe = (L.h + R.h) / 2.0;
  const double uRoe = (sL * uL + sR * uR) / (sL + sR);
  const double vRoe = (sL * vL + sR * vR) / (sL + sR);
  const double unRoe = uRoe * nx + vRoe * ny;
  const double cRoe = smooth_sqrt(g * hRoe);
  const double o2c = 0.5 / cRoe;
  const double d1 = R.hu - L.hu, d2 = R.hv - L.hv;
  double w0 = -(uRoe * ny - vRoe * nx) * dxi + ny * d1 + (-nx) * d2;
  double w1 = (unRoe * o2c + 0.5) * dxi + (-nx * o2c) * d1 + (-ny * o2c) * d2;
  double w2 = (-unRoe * o2c + 0.5) * dxi + (nx * o2c) * d1 + (ny * o2c) * d2;
  w0 *= smooth_abs(unRoe);
  w1 *= smooth_abs(unRoe - cRoe);
  w2 *= smooth_abs(unRoe + cRoe);
  const double A0 = w1 + w2;
  const double A1 = ny * w0 + (uRoe - cRoe * nx) * w1 + (uRoe + cRoe * nx) * w2;
  const double A2 = (-nx) * w0 + (vRoe - cRoe * ny) * w1 + (vRoe + cRoe * ny) * w2;
  const double pR = 0.5 * g * (smooth_pow2(R.xi) + 2.0 * R.xi * R.hst);
  const double fL0 = L.hu * nx + L.hv * ny;
  const double fL1 = o.hu_uL_pL * nx + o.hu_vL * ny;
  const double fL2 = o.hv_uL * nx + o.hv_vL_pL * ny;
  const double fR0 = R.hu * nx + R.hv * ny;
  const double fR1 = (R.hu * uR + pR) * nx + R.hu * vR * ny;
  const double fR2 = (R.hv * uR) * nx + (R.hv * vR + pR) * ny;
  F[0] = (fL0 + fR0 - A0) / 2.0;
  F[1] = (fL1 + fR1 - A1) / 2.0;
  F[2] = (fL2 + fR2 - A2) / 2.0;
}

// Sum over faces of F * L for cell c (FP64).
__device__ __forceinline__ void face_sum_f64(const DevMesh& m, const double* __restrict__ Q, int c,
                                             const Side<double>& L, double& f0, double& f1, double& f2) {
  f0 = 0.0; f1 = 0.0; f2 = 0.0;
  OwnF64 own;
  if (!L.dry) own = own_f64(L, m.g);
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * m.n + c];
    if (nb == kNoFace) break;
    const double nx = m.snx[(size_t)k * m.n + c], ny = m.sny[(size_t)k * m.n + c];
    const double len = m.slen[(size_t)k * m.n + c];
    Side<double> R;
    if (nb >= 0) {
      R = load_f64(m, Q, nb);
    } else {
      const int32_t bf = boundary_index(nb);
      const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
      R = ghost_state<double>(L, type, nx, ny, m.hsm, type == kBcExitH ? m.exitWse[grp] : 0.0,
                              type == kBcInletQ ? m.inletQ[grp] : 0.0, type == kBcInletQ ? m.totalA[grp] : 1.0,
                              m.bfLp23[bf], m.man[c]);
    }
    double F[3];
    if (m.riemann == kRiemannHll) hll_flux<double>(L, R, R.xi - L.xi, m.g, nx, ny, m.hsm, F);
    else if (!L.dry && !R.dry) roe_flux_wet_f64(L, own, R, R.xi - L.xi, m.g, nx, ny, F);
    else roe_flux<double>(L, R, R.xi - L.xi, m.g, nx, ny, m.hsm, F);
    f0 = f0 + F[0] * len;
    f1 = f1 + F[1] * len;
    f2 = f2 + F[2] * len;
  }
}

// CFL candidate A / sum_f L (|u.n| + sqrt(g h)) of one cell.
__device__ __forceinline__ double cfl_candidate_f64(const DevMesh& m, int c, double xi, double qx, double qy) {
  double h = xi + m.hst[c];
  if (h <= m.hsm) { h = m.hsm; qx = 0.0; qy = 0.0; }
  const double u = qx / h, v = qy / h, a = sqrt(m.g * h);
  double s = 0.0;
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * m.n + c];
    if (nb == kNoFace) break;
    s += m.slen[(size_t)k * m.n + c] * (fabs(u * m.snx[(size_t)k * m.n + c] + v * m.sny[(size_t)k * m.n + c]) + a);
  }
  return m.area[c] / s;
}

__global__ void __launch_bounds__(kBlock) k_stage_f64(DevMesh m, DevScalars s, int mode, const double* __restrict__ Qin,
                                                      const double* Qbase, double* Qout, int cfl) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = c < m.n;
  double cand = INFINITY;
  const int mem = (s.nMembers > 0 && active) ? member_of(s, c) : -1;   // an ensemble member's own step
  if (active) {
    const Side<double> L = load_f64(m, Qin, c);
    double f0, f1, f2;
    face_sum_f64(m, Qin, c, L, f0, f1, f2);
    const double A = m.area[c];
    const double r0 = -f0 / A, r1 = -f1 / A, r2 = -f2 / A;     // :415
    // Sources (:449-559): (h > h_small) * (g xi S0 - friction), continuity 0.
    // Manning friction, or the flow-resistance closure F q / |q|_smooth
    // (semi_discretize_swe_2D.jl:517-529) with F from the resistance kernels.
    double fx, fy;
    if (m.res.kind == kResUdeFlowResistance) {
      const double mag = smooth_sqrt(L.hu * L.hu + L.hv * L.hv);
      fx = m.res.fres[c] * L.hu / mag;
      fy = m.res.fres[c] * L.hv / mag;
    } else {
      const double fr = friction_coef(m.g, m.kn2, m.hsm, m.man[c], L.h, L.hu, L.hv);
      fx = fr * L.hu;
      fy = fr * L.hv;
    }
    const double sx = L.dry ? 0.0 : (m.g * L.xi * m.s0x[c] - fx);
    const double sy = L.dry ? 0.0 : (m.g * L.xi * m.s0y[c] - fy);
    const double d0 = r0 + 0.0, d1 = r1 + sx, d2 = r2 + sy;
    if (mode == kModeRhs) {
      Qout[c] = d0; Qout[m.n + c] = d1; Qout[2 * m.n + c] = d2;
    } else {
      const double dt = mem >= 0 ? s.dtM[mem] : *s.dt;
      double x0, x1, x2;
      if (mode == kModeStage2) {
        x0 = 0.5 * (Qbase[c] + (Qin[c] + dt * d0));
        x1 = 0.5 * (Qbase[m.n + c] + (Qin[m.n + c] + dt * d1));
        x2 = 0.5 * (Qbase[2 * m.n + c] + (Qin[2 * m.n + c] + dt * d2));
      } else {
        x0 = Qin[c] + dt * d0;
        x1 = Qin[m.n + c] + dt * d1;
        x2 = Qin[2 * m.n + c] + dt * d2;
      }
      if (mode == kModeEulerRef) {
        // custom_ODE_update_cells (custom_ODE_solvers.jl:18-26): first block compared as if it were h.
        if (x0 < m.hsm) { x0 = m.hsm; x1 = 0.0; x2 = 0.0; }
      } else if (x0 + m.hst[c] <= m.hsm) {
        // depth-positivity clamp: the cell is dry, h = h_small, q = 0
        x0 = dry_xi(m.hsm, m.hst[c]); x1 = 0.0; x2 = 0.0;
      }
      if (!(isfinite(x0) && isfinite(x1) && isfinite(x2))) atomicOr(s.flags, 1);
      Qout[c] = x0; Qout[m.n + c] = x1; Qout[2 * m.n + c] = x2;
      if (cfl) cand = cfl_candidate_f64(m, c, x0, x1, x2);
    }
  }
  if (cfl && s.nMembers > 0) member_min_publish(s, cand, mem);
  else if (cfl) block_min_publish(cand, s.cflMin);
}

__global__ void __launch_bounds__(kBlock) k_cfl_f64(DevMesh m, DevScalars s, const double* __restrict__ Q) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double cand = INFINITY;
  if (c < m.n) cand = cfl_candidate_f64(m, c, Q[c], Q[m.n + c], Q[2 * m.n + c]);
  if (s.nMembers > 0) member_min_publish(s, cand, c < m.n ? member_of(s, c) : -1);
  else block_min_publish(cand, s.cflMin);
}

// total_A = sum_faces L^(5/3) h / n * wet over one inlet-Q boundary (bc_2D.jl:673-679).
__global__ void __launch_bounds__(kBlock) k_inlet_total_f64(DevMesh m, DevScalars s, const double* __restrict__ Q) {
  const int g = blockIdx.x;
  const int o0 = m.inletOff[g], o1 = m.inletOff[g + 1];
  double acc = 0.0;
  for (int i = o0 + threadIdx.x; i < o1; i += blockDim.x) {
    const int c = m.inletCell[i];
    const Side<double> L = load_f64(m, Q, c);
    acc += L.dry ? 0.0 : m.inletLp53[i] * L.h / m.man[c] * 1.0;
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) {
    m.totalA[g] = t;
    if (!(t > 1e-10)) atomicOr(s.flags, 2);
  }
}

}  // namespace

namespace {
// Hydrographs: one thread per inlet-Q group (see DevMesh::hydroOff).
__global__ void k_hydrograph(DevMesh m, DevScalars s, int when, double t) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.nInlet) return;
  const int a = m.hydroOff[g], b = m.hydroOff[g + 1];
  if (b <= a) return;   // constant discharge
  if (s.nMembers > 0 && s.inletMember && when != kHydroAt) {   // an ensemble: the group's member's own time
    const int mm = s.inletMember[g];
    t = when == kHydroStepStart ? s.tM[mm] - s.dtM[mm] : s.tM[mm];
  } else if (when == kHydroStepStart) {
    t = *s.tSum - *s.dt;
  } else if (when == kHydroStepEnd || when == kHydroNow) {
    t = *s.tSum;
  }
  double q;
  if (t <= m.hydroT[a]) {
    q = m.hydroQ[a];
  } else if (t >= m.hydroT[b - 1]) {
    q = m.hydroQ[b - 1];
  } else {
    int k = a;
    while (k + 1 < b - 1 && m.hydroT[k + 1] <= t) ++k;   // bounded by the group's points
    const double w = (t - m.hydroT[k]) / (m.hydroT[k + 1] - m.hydroT[k]);
    q = m.hydroQ[k] + w * (m.hydroQ[k + 1] - m.hydroQ[k]);
  }
  const_cast<double*>(m.inletQ)[g] = q;
}

}  // namespace

int launch_hydrograph(const DevMesh& m, const DevScalars& s, int when, double t, cudaStream_t st) {
  if (m.nHydro == 0 || m.nInlet == 0) return 0;
  k_hydrograph<<<(m.nInlet + 31) / 32, 32, 0, st>>>(m, s, when, t);
  return 1;
}

void launch_inlet_total_f64(const DevMesh& m, const DevScalars& s, const double* Q, cudaStream_t st) {
  launch_resistance_f64(m, Q, st);
  if (m.nInlet > 0) k_inlet_total_f64<<<m.nInlet, kBlock, 0, st>>>(m, s, Q);
}
// Block size of the FP64 stage: 256 threads, halved (down to one warp) while
// the grid would give fewer than 4 blocks per SM -- on a small mesh the
// FP64-bound kernel then spreads over every SM instead of a few.  A cell's
// result does not depend on the block it runs in (the CFL minimum is exact).
int stage_block_f64(int n) {
  static const int sms = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  int bs = kBlock;
  while (bs > 32 && (n + bs - 1) / bs < 4 * sms) bs /= 2;
  return bs;
}

void launch_stage_f64(const DevMesh& m, const DevScalars& s, int mode, const double* Qin, const double* Qbase,
                      double* Qout, bool cfl, cudaStream_t st) {
  const int bs = stage_block_f64(m.n);
  k_stage_f64<<<(m.n + bs - 1) / bs, bs, 0, st>>>(m, s, mode, Qin, Qbase, Qout, cfl ? 1 : 0);
}
void launch_cfl_f64(const DevMesh& m, const DevScalars& s, const double* Q, cudaStream_t st) {
  k_cfl_f64<<<blocks_for(m.n), kBlock, 0, st>>>(m, s, Q);
}

}  // namespace hg
