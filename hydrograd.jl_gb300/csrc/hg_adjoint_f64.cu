// Adjoint (vector-Jacobian product) kernels of the FP64 path.
//
// For the RHS R_c = -(1/A_c) sum_f F(U_c, U_nb(f)) L_f + S_c(U_c) of
// semi_discretize_swe_2D.jl:286-559, cell j gathers
//   (J^T mu)_j = sum_f (dF(U_j, U_nb)/dU_j)^T L_f (mu_nb/A_nb - mu_j/A_j)    (interior faces)
//              + sum_f (dF(U_j, G(U_j))/dU_j)^T (-L_f mu_j/A_j)               (boundary faces)
//              + (dS_j/dU_j)^T mu_j
// using F(U_nb, U_j, -n) = -F(U_j, U_nb, n), which holds branch by branch for
// the Roe flux with its dry/wet cases (swe_2D_solvers.jl:16-76 mirror each
// other).  U_j = (xi, h, hu, hv) with the clamp of semi_discretize_swe_2D.jl:
// 101-106 (a dry cell's h and q do not depend on Q).  The local Jacobians come
// from the forward code itself evaluated on dual numbers (hg_dual.cuh), so
// every branch is the forward pass's.  No atomics: every output element is
// written by the thread of its cell.
#include <cfloat>
#include <cmath>

#include "hg_adjoint_state.hpp"
#include "hg_device.cuh"
#include "hg_dual.cuh"
#include "hg_reduce.cuh"
#include "hg_resfn.cuh"
#include "hg_wet_vjp.cuh"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = 128;
inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

using D3 = Dn<double, 3>;   // xi, qx, qy of the cell
using D7 = Dn<double, 7>;   // + Manning n, zb, inlet Q, inlet total_A (boundary faces)

__device__ __forceinline__ Side<double> load_side(const DevMesh& m, const double* __restrict__ Q, int j) {
  Side<double> s;
  s.xi = Q[j];
  s.hst = m.hst[j];
  s.zb = m.zb[j];
  const double h = s.xi + s.hst;
  s.dry = h <= m.hsm;
  s.h = s.dry ? m.hsm : h;
  s.hu = s.dry ? 0.0 : Q[m.n + j];
  s.hv = s.dry ? 0.0 : Q[2 * m.n + j];
  return s;
}

template <class D>
__device__ __forceinline__ Side<D> seeded(const Side<double>& s, int kzb) {
  Side<D> r;
  r.xi = D::seed(s.xi, 0);
  r.hst = D(s.hst);
  r.zb = D::seed(s.zb, kzb);
  r.dry = s.dry;
  r.h = s.dry ? D(s.h) : D::seed(s.h, 0);
  r.hu = s.dry ? D(0.0) : D::seed(s.hu, 1);
  r.hv = s.dry ? D(0.0) : D::seed(s.hv, 2);
  return r;
}

template <class D>
__device__ __forceinline__ Side<D> constant(const Side<double>& s) {
  Side<D> r;
  r.xi = D(s.xi); r.hst = D(s.hst); r.zb = D(s.zb); r.dry = s.dry;
  r.h = D(s.h); r.hu = D(s.hu); r.hv = D(s.hv);
  return r;
}

__global__ void __launch_bounds__(kBlock) k_vjp_f64(DevMesh m, AdjDev a, const double* __restrict__ Q,
                                                    const double* __restrict__ mu, const double* __restrict__ extra,
                                                    double* out, double cSelf, double cExtra, double beta,
                                                    int useMask) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m.n) return;
  const int n = m.n;
  const Side<double> L = load_side(m, Q, j);
  const double Aj = m.area[j];
  const double mj0 = mu[j], mj1 = mu[n + j], mj2 = mu[2 * n + j];
  double g0 = 0.0, g1 = 0.0, g2 = 0.0, gn = 0.0, gzb = 0.0, gF = 0.0;
  const Side<D3> L3 = seeded<D3>(L, -1);
  // Interior wet-wet faces in reverse mode (hg_wet_vjp.cuh); faces with a dry
  // side through 3-direction duals of the reference solver.
  const bool wetL = !L.dry;
  OwnV<double> own;
  if (wetL) own = own_v(L);
  OwnAdj<double> bo;
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * n + j];
    if (nb == kNoFace) break;
    const double nx = m.snx[(size_t)k * n + j], ny = m.sny[(size_t)k * n + j];
    const double len = m.slen[(size_t)k * n + j];
    if (nb >= 0) {
      const Side<double> R = load_side(m, Q, nb);
      const double An = m.area[nb];
      const double w0 = len * (mu[nb] / An - mj0 / Aj);
      const double w1 = len * (mu[n + nb] / An - mj1 / Aj);
      const double w2 = len * (mu[2 * n + nb] / An - mj2 / Aj);
      if (wetL && !R.dry && m.riemann == kRiemannRoe) {
        roe_wet_vjp<double>(L, own, R, R.xi - L.xi, m.g, nx, ny, w0, w1, w2, bo);
        continue;
      }
      const Side<D3> R3 = constant<D3>(R);
      D3 F[3];
      riemann_flux<D3>(m.riemann, L3, R3, R3.xi - L3.xi, D3(m.g), D3(nx), D3(ny), D3(m.hsm), F);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double c = w0 * F[0].d[d] + w1 * F[1].d[d] + w2 * F[2].d[d];
        if (d == 0) g0 += c; else if (d == 1) g1 += c; else g2 += c;
      }
    } else {
      const int32_t bf = boundary_index(nb);
      const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
      const double w0 = -len * mj0 / Aj, w1 = -len * mj1 / Aj, w2 = -len * mj2 / Aj;
      const Side<D7> L7 = seeded<D7>(L, 4);
      const D7 man = D7::seed(m.man[j], 3);
      const D7 qin = D7::seed(type == kBcInletQ ? m.inletQ[grp] : 0.0, 5);
      const D7 ta = D7::seed(type == kBcInletQ ? m.totalA[grp] : 1.0, 6);
      const Side<D7> R7 = ghost_state<D7>(L7, type, D7(nx), D7(ny), D7(m.hsm),
                                          D7(type == kBcExitH ? m.exitWse[grp] : 0.0), qin, ta, D7(m.bfLp23[bf]), man);
      D7 F[3];
      riemann_flux<D7>(m.riemann, L7, R7, R7.xi - L7.xi, D7(m.g), D7(nx), D7(ny), D7(m.hsm), F);
      double c[7];
#pragma unroll
      for (int d = 0; d < 7; ++d) c[d] = w0 * F[0].d[d] + w1 * F[1].d[d] + w2 * F[2].d[d];
      g0 += c[0]; g1 += c[1]; g2 += c[2];
      gn += c[3];
      gzb += c[4];
      a.bfGradQ[bf] = c[5];
      a.bfGradTA[bf] = c[6];
    }
  }
  if (wetL) {
    double gx, gu, gv;
    own_vjp<double>(L, own, m.g, bo, gx, gu, gv);
    g0 += gx;
    g1 += gu;
    g2 += gv;
  }
  // Sources (semi_discretize_swe_2D.jl:449-559), wet cells only.
  if (!L.dry) {
    // friction k q: Manning k = g n^2 |q| / (kn^2 hp^(7/3)), or the
    // flow-resistance closure's k = F / |q| (|q| smoothed as in the RHS)
    const double s = sqrt(L.hu * L.hu + L.hv * L.hv + eps_c<double>());
    double k, dkdh, dkdqx, dkdqy;
    if (m.res.kind == kResUdeFlowResistance) {
      k = m.res.fres[j] / s;
      dkdh = 0.0;
      dkdqx = -k * L.hu / (s * s);
      dkdqy = -k * L.hv / (s * s);
      gF = -(mj1 * L.hu + mj2 * L.hv) / s;
    } else {
      const double hp = L.h + m.hsm;
      k = m.g * (m.man[j] * m.man[j]) / m.kn2 / (hp * hp * cbrt(hp)) * s;   // as friction_coef
      dkdh = -(7.0 / 3.0) * k / hp;
      dkdqx = k * L.hu / (s * s);
      dkdqy = k * L.hv / (s * s);
      gn += -(mj1 * L.hu + mj2 * L.hv) * (2.0 * k / m.man[j]);
    }
    g0 += mj1 * (m.g * m.s0x[j] - L.hu * dkdh) + mj2 * (m.g * m.s0y[j] - L.hv * dkdh);
    g1 += mj1 * (-k - L.hu * dkdqx) + mj2 * (-L.hv * dkdqx);
    g2 += mj1 * (-L.hu * dkdqy) + mj2 * (-k - L.hv * dkdqy);
    a.gS0x[j] += beta * mj1 * m.g * L.xi;
    a.gS0y[j] += beta * mj2 * m.g * L.xi;
  }
  if (a.resChain) {   // n = f(state): dL/dn into the state and the function's parameters
    if (gn != 0.0) {
      const ResJac<double> J = manning_jac<double>(m.res, L.h, L.hu, L.hv, m.res.ks ? m.res.ks[j] : 0.0, L.dry);
      g0 += gn * J.dh;
      g1 += gn * J.dqx;
      g2 += gn * J.dqy;
#pragma unroll
      for (int k = 0; k < 4; ++k) a.gResP[(size_t)k * n + j] += beta * gn * J.dp[k];
    }
  } else if (a.udeChain == 1) {   // n from the network: the network's VJP takes it on
    a.udeGn[j] = beta * gn;
  } else {
    a.gN[j] += beta * gn;
  }
  if (a.udeChain == 2) a.udeGn[j] = beta * gF;   // F of the flow-resistance closure
  a.gZb[j] += beta * gzb;
  // the stage clamp zeroes the derivative of a dry cell (useMask = 0: a state
  // no clamp produced, e.g. a Tsit5 stage)
  const double mask = (useMask && L.dry) ? 0.0 : 1.0;
  const double e0 = extra ? extra[j] : 0.0, e1 = extra ? extra[n + j] : 0.0, e2 = extra ? extra[2 * n + j] : 0.0;
  out[j] = mask * (cSelf * mj0 + cExtra * e0 + beta * g0);
  out[n + j] = mask * (cSelf * mj1 + cExtra * e1 + beta * g1);
  out[2 * n + j] = mask * (cSelf * mj2 + cExtra * e2 + beta * g2);
}

// total_A_b = sum_faces L^(5/3) h_i / n_i wet_i (bc_2D.jl:673-676): its adjoint
// gTA_b = sum over the group's boundary faces of w . dF/dtotal_A is spread back
// to the group's cells.  One block per group, one thread per distinct cell.
__global__ void __launch_bounds__(256) k_inlet_adjoint_f64(DevMesh m, AdjDev a, const double* __restrict__ Q,
                                                           double* out, double beta, int g) {
  const int o0 = m.inletOff[g], o1 = m.inletOff[g + 1];
  double sTA = 0.0, sQ = 0.0;
  for (int i = o0 + threadIdx.x; i < o1; i += blockDim.x) {
    const int bf = a.inletBf[i];
    sTA += a.bfGradTA[bf];
    sQ += a.bfGradQ[bf];
  }
  __shared__ double tot[2];
  const double t1 = block_sum(sTA);
  if (threadIdx.x == 0) tot[0] = t1;
  const double t2 = block_sum(sQ);
  if (threadIdx.x == 0) {
    tot[1] = t2;
    a.gQ[g] += beta * t2;
  }
  __syncthreads();
  const double gTA = tot[0];
  const int u0 = a.inletUOff[g], u1 = a.inletUOff[g + 1];
  for (int i = u0 + threadIdx.x; i < u1; i += blockDim.x) {
    const int c = a.inletUCell[i];
    const Side<double> L = load_side(m, Q, c);
    if (L.dry) continue;                      // wet_i = 0, and the clamp zeroes a dry cell's derivative
    const double coef = a.inletUCoef[i], n = m.man[c];
    out[c] += beta * gTA * coef / n;          // d total_A / d xi_c (h = xi + hstill)
    const double gn = gTA * (-coef * L.h / (n * n));
    if (a.resChain && gn != 0.0) {   // n = f(state): into the state and the function's parameters
      const ResJac<double> J = manning_jac<double>(m.res, L.h, L.hu, L.hv, m.res.ks ? m.res.ks[c] : 0.0, false);
      const int N = m.n;
      out[c] += beta * gn * J.dh;
      out[N + c] += beta * gn * J.dqx;
      out[2 * N + c] += beta * gn * J.dqy;
      for (int k = 0; k < 4; ++k) a.gResP[(size_t)k * N + c] += beta * gn * J.dp[k];
    } else if (a.udeChain == 1) {
      a.udeGn[c] += beta * gn;
    } else if (!a.resChain) {
      a.gN[c] += beta * gn;
    }
  }
}

__global__ void __launch_bounds__(256) k_probe_loss_f64(DevMesh m, AdjDev a, const double* __restrict__ Q,
                                                        const int32_t* __restrict__ probes,
                                                        const double* __restrict__ obs, int np) {
  double s = 0.0;
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    const int c = probes[p];
    const double e = (Q[c] + m.hst[c]) - obs[p];
    s += e * e;
  }
  const double t = block_sum(s);
  if (threadIdx.x == 0) a.loss[0] += t;
}

__global__ void k_probe_adjoint_f64(DevMesh m, const double* __restrict__ Q, double* mu,
                                    const int32_t* __restrict__ probes, const double* __restrict__ obs, int np,
                                    double scale, int useMask) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int p = 0; p < np; ++p) {              // sequential: a probe cell listed twice adds twice, in order
    const int c = probes[p];
    const double h = Q[c] + m.hst[c];
    if (useMask && h <= m.hsm) continue;      // clamped at the step's output: derivative 0
    mu[c] += scale * 2.0 * (h - obs[p]);
  }
}

// dL/dzb_j = sum_f of the transposed S0 = -GreenGauss(zb_faces) map
// (process_bed_2D.jl:46-66; fvm_schemes_2D.jl:197-213,253-275) + the direct term.
// dL/dS0 / A per cell, in place (the gradient w.r.t. S0 is not needed after
// this), so that k_zb_gradient divides once per cell rather than once per face.
__global__ void __launch_bounds__(256) k_zb_scale(DevMesh m, AdjDev a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m.n) return;
  a.gS0x[j] = a.gS0x[j] / m.area[j];
  a.gS0y[j] = a.gS0y[j] / m.area[j];
}

__global__ void __launch_bounds__(256) k_zb_gradient(DevMesh m, AdjDev a, double* gzb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m.n) return;
  const int n = m.n;
  const double gxj = a.gS0x[j], gyj = a.gS0y[j];
  double acc = a.gZb[j];
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * n + j];
    if (nb == kNoFace) break;
    const double nx = m.snx[(size_t)k * n + j], ny = m.sny[(size_t)k * n + j];
    const double len = m.slen[(size_t)k * n + j];
    if (nb >= 0) {
      const double gxn = a.gS0x[nb], gyn = a.gS0y[nb];
      acc += -0.5 * len * ((gxj - gxn) * nx + (gyj - gyn) * ny);
    } else {
      acc += -len * (gxj * nx + gyj * ny);
    }
  }
  gzb[j] = acc;
}

}  // namespace

void launch_vjp_f64(const DevMesh& m, const AdjDev& a, const double* Q, const double* mu, const double* extra,
                    double* out, double cSelf, double cExtra, double beta, cudaStream_t st, bool mask) {
  // at most the kernel's launch bound; a cell's result does not depend on its block
  const int bs = stage_block_f64(m.n) < kBlock ? stage_block_f64(m.n) : kBlock;
  k_vjp_f64<<<(m.n + bs - 1) / bs, bs, 0, st>>>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, mask ? 1 : 0);
}
void launch_inlet_adjoint_f64(const DevMesh& m, const AdjDev& a, const double* Q, double* out, double beta,
                              cudaStream_t st) {
  for (int g = 0; g < m.nInlet; ++g) k_inlet_adjoint_f64<<<1, 256, 0, st>>>(m, a, Q, out, beta, g);
}
void launch_probe_loss_f64(const DevMesh& m, const AdjDev& a, const double* Q, const int32_t* probes,
                           const double* obs, int32_t nprobe, cudaStream_t st) {
  if (nprobe > 0) k_probe_loss_f64<<<1, 256, 0, st>>>(m, a, Q, probes, obs, nprobe);
}
void launch_probe_adjoint_f64(const DevMesh& m, const double* Q, double* mu, const int32_t* probes,
                              const double* obs, int32_t nprobe, double scale, cudaStream_t st, bool mask) {
  if (nprobe > 0) k_probe_adjoint_f64<<<1, 32, 0, st>>>(m, Q, mu, probes, obs, nprobe, scale, mask ? 1 : 0);
}
namespace {
// The gradient w.r.t. the parameters of a state-dependent n: the per-cell
// sums added over all cells, one block per parameter in a fixed order.
__global__ void __launch_bounds__(256) k_res_param_sum(AdjDev a, int n, double* out4) {
  const int k = blockIdx.x;
  double s = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) s += a.gResP[(size_t)k * n + j];
  const double t = block_sum(s);
  if (threadIdx.x == 0) out4[k] = t;
}
}  // namespace

void launch_res_param_sum(const AdjDev& a, int n, double* out4, cudaStream_t st) {
  k_res_param_sum<<<4, 256, 0, st>>>(a, n, out4);
}

void launch_zb_gradient(const DevMesh& m, const AdjDev& a, double* gzb, cudaStream_t st) {
  k_zb_scale<<<(m.n + 255) / 256, 256, 0, st>>>(m, a);
  k_zb_gradient<<<(m.n + 255) / 256, 256, 0, st>>>(m, a, gzb);
}

}  // namespace hg
