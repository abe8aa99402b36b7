// Adjoint (vector-Jacobian product) kernels of the FP32-compensated path.
//
// Same gather-form VJP as hg_adjoint_f64.cu (see there for the formulas), on
// the packed FP32 records (hg_f32.cuh), with the FP32 path's own wet/dry
// decisions (depth_f32) so that every branch is the forward pass's.
// Cotangents are FP32; per-cell parameter gradients accumulate as compensated
// FP32 pairs (GB300's FP64 rate is a small fraction of its FP32 rate) and are
// folded into FP64 once, after the reverse sweep.
// Compiled with the same fast-math options as the FP32 forward kernels.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "hg_adjoint_state.hpp"
#include "hg_async.cuh"
#include "hg_device.cuh"
#include "hg_dual.cuh"
#include "hg_f32.cuh"
#include "hg_pdl.cuh"
#include "hg_reduce.cuh"
#include "hg_resfn.cuh"
#include "hg_wet_vjp.cuh"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = 128;
inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

using F3 = Dn<float, 3>;
using F7 = Dn<float, 7>;

template <class D>
__device__ __forceinline__ Side<D> seeded(const Side<float>& s, int kzb) {
  Side<D> r;
  r.xi = D::seed(s.xi, 0);
  r.hst = D(s.hst);
  r.zb = D::seed(s.zb, kzb);
  r.dry = s.dry;
  r.h = s.dry ? D(s.h) : D::seed(s.h, 0);
  r.hu = s.dry ? D(0.0f) : D::seed(s.hu, 1);
  r.hv = s.dry ? D(0.0f) : D::seed(s.hv, 2);
  return r;
}

template <class D>
__device__ __forceinline__ Side<D> constant(const Side<float>& s) {
  Side<D> r;
  r.xi = D(s.xi); r.hst = D(s.hst); r.zb = D(s.zb); r.dry = s.dry;
  r.h = D(s.h); r.hu = D(s.hu); r.hv = D(s.hv);
  return r;
}

// acc += b * g with the product exact (fma residual) and the sum compensated:
// FP32 instructions only, about 2^-44 relative over thousands of terms.
__device__ __forceinline__ void acc_add_from(float2* p, float2 a, float b, float g) {
  const float prod = b * g;
  const float perr = fmaf(b, g, -prod);
  float s, e;
  two_sum(a.x, prod, s, e);
  e += a.y + perr;
  fast_two_sum(s, e, a.x, a.y);
  *p = a;
}
__device__ __forceinline__ void acc_add(float2* p, float b, float g) { acc_add_from(p, *p, b, g); }

// The accumulators a VJP cell updates from its own values (q: 0 n, 1 S0x,
// 2 S0y), prefetched with the tile where the kernel is pipelined.
__device__ __forceinline__ bool acc_prefetched(const AdjDev& a, int q) {
  return q == 0 ? (a.wantN && !a.resChain && !a.udeChain) : a.wantZb != 0;
}

// Interior faces (3-direction duals: d/d own xi, hu, hv) and the source
// terms.  Boundary faces, whose ghost states also depend on n, zb, Q and
// total_A (7-direction duals), are added afterwards by k_vjp_bnd_f32, so that
// this kernel -- the one over every cell -- carries only the registers of the
// 3-direction flux.
template <int NS>
constexpr int vjp_min_blocks() { return NS <= 4 ? 5 : 1; }   // <= 96 registers, no spills

// Where a VJP reads its data: the cell's own records and cotangents, its slot
// records, and a neighbour's records and cotangents.  GlobalSrc reads device
// memory (neighbours by cell id); TileSrc a pipelined tile in shared memory
// (neighbours by tile-local index: own cells, then the tile's halo).
struct VjpNbr {
  float4 x, p;
  float area, m0, m1, m2;
};
struct GlobalSrc {
  const DevMesh& m;
  StateF32 Q;
  const float* mu;
  const float* extra;
  int j;
  __device__ float4 x() const { return __ldg(&Q.x[j]); }
  __device__ float4 cp() const { return __ldg(&m.CP[j]); }
  __device__ float4 cs() const { return __ldg(&m.CS[j]); }
  __device__ float mu_own(int b) const { return mu[(size_t)b * m.n + j]; }
  __device__ float extra_own(int b) const { return extra ? extra[(size_t)b * m.n + j] : 0.0f; }
  __device__ float4 slot(int k) const { return __ldg(&m.SL[(size_t)k * m.n + j]); }
  __device__ VjpNbr nbr(int nb) const {
    return VjpNbr{__ldg(&Q.x[nb]), __ldg(&m.CP[nb]), __ldg(&m.CS[nb]).z, mu[nb], mu[m.n + nb],
                  mu[2 * (size_t)m.n + nb]};
  }
  __device__ int cell(int nb) const { return nb; }   // the neighbour's cell id
  __device__ float2 acc(int, const float2* p) const { return *p; }
};

// The VJP of one stage at cell j (interior faces: 3-direction duals of the
// reference solver where a side is dry, reverse mode where both are wet; the
// sources), written to out[j] and the cell's parameter accumulators.  FOLD:
// the boundary faces too, from their flux Jacobians (a.bndJ), and the inlet
// conveyance terms with the groups' total_A cotangents grpTA.
// NOMASK: the VJP of the RHS alone (the stages of a Tsit5 step, which no clamp
// of the stage state follows): a dry cell's output is not masked, and its
// interior faces, through which the RHS depends on the cell's own xi, are
// differentiated by the dual-number path.
template <int NS, bool FOLD, class Src, bool NOMASK = false>
__device__ __forceinline__ void vjp_cell(const DevMesh& m, const AdjDev& a, int j, const Src& src, float* out,
                                         float cSelf, float cExtra, float beta, const double* grpTA = nullptr) {
  const int n = m.n;
  const float4 cp = src.cp();
  const float4 cs = src.cs();
  const SideF32 L = make_side_f32(src.x(), cp, m.hsmf, m.hsmLo);
  const float Aj = cs.z;
  const float mj0 = src.mu_own(0), mj1 = src.mu_own(1), mj2 = src.mu_own(2);
  float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gn = 0.0f;
  unsigned int bnd = 0u;   // FOLD: the slots that hold boundary faces
  if (!L.s.dry || NOMASK) {   // (masked: a dry cell's output is zero, and its faces add to nothing else)
    // Wet-wet faces in reverse mode (roe_wet_vjp, the own quantities'
    // adjoints summed over the faces and taken back once); faces with a dry
    // neighbour through 3-direction duals of the reference solver.
    const OwnV<float> o = own_v(L.s);
    OwnAdj<float> b;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const float4 sl = src.slot(k);
      const int32_t nb = slot_nb(sl);
      if (nb < 0) {   // no face, or a boundary face (folded below, or k_vjp_bnd_f32)
        if (FOLD && nb != kNoFace) bnd |= 1u << k;
        continue;
      }
      const float nx = sl.x, ny = sl.y, len = sl.z;
      const VjpNbr r = src.nbr(nb);
      const SideF32 R = make_side_f32(r.x, r.p, m.hsmf, m.hsmLo);
      const float An = r.area;
      const float w0 = len * (r.m0 / An - mj0 / Aj);
      const float w1 = len * (r.m1 / An - mj1 / Aj);
      const float w2 = len * (r.m2 / An - mj2 / Aj);
      if (!L.s.dry && !R.s.dry && m.riemann == kRiemannRoe) {
        roe_wet_vjp<float>(L.s, o, R.s, (R.s.xi - L.s.xi) + (R.xlo - L.xlo), m.gf, nx, ny, w0, w1, w2, b);
      } else {
        const Side<F3> L3 = seeded<F3>(L.s, -1);
        const Side<F3> R3 = constant<F3>(R.s);
        const F3 dxi = (R3.xi - L3.xi) + F3(R.xlo - L.xlo);
        // the forward pass's wall test (bank_wall_f64), so that the same branch is differentiated
        int bank = -1;
        if (R.s.dry && !L.s.dry) bank = bank_wall_f64(m, L.s.xi, L.xlo, j, src.cell(nb));
        else if (NOMASK && L.s.dry && !R.s.dry) bank = bank_wall_f64(m, R.s.xi, R.xlo, src.cell(nb), j);
        F3 F[3];
        riemann_flux<F3>(m.riemann, L3, R3, dxi, F3(m.gf), F3(nx), F3(ny), F3(m.hsmf), F, bank);
        g0 += w0 * F[0].d[0] + w1 * F[1].d[0] + w2 * F[2].d[0];
        g1 += w0 * F[0].d[1] + w1 * F[1].d[1] + w2 * F[2].d[1];
        g2 += w0 * F[0].d[2] + w1 * F[1].d[2] + w2 * F[2].d[2];
      }
    }
    if (!L.s.dry) {   // (a dry cell -- NOMASK -- has no wet-wet face and no source term)
    float gx, gu, gv;
    own_vjp<float>(L.s, o, m.gf, b, gx, gu, gv);
    g0 += gx;
    g1 += gu;
    g2 += gv;
    // friction k q: Manning, or the flow-resistance closure's k = F / |q|
    const float hu = L.s.hu, hv = L.s.hv, man = cp.w;
    const float s2 = hu * hu + hv * hv + eps_c<float>();
    float k, dkdh, dkdqx, dkdqy;
    if (m.res.kind == kResUdeFlowResistance) {
      const float s = sqrtf(s2);
      k = m.res.fresF[j] / s;
      dkdh = 0.0f;
      dkdqx = -k * hu / s2;
      dkdqy = -k * hv / s2;
      gn = -(mj1 * hu + mj2 * hv) / s;   // dL/dF (no term of the interior faces depends on n)
    } else {
      const float hp = L.s.h + m.hsmf;
      k = friction_coef(m.gf, m.kn2f, m.hsmf, man, L.s.h, hu, hv);
      dkdh = -(7.0f / 3.0f) * k / hp;
      dkdqx = k * hu / s2;
      dkdqy = k * hv / s2;
      gn += -(mj1 * hu + mj2 * hv) * (2.0f * k / man);
    }
    g0 += mj1 * (m.gf * cs.x - hu * dkdh) + mj2 * (m.gf * cs.y - hv * dkdh);
    g1 += mj1 * (-k - hu * dkdqx) + mj2 * (-hv * dkdqx);
    g2 += mj1 * (-hu * dkdqy) + mj2 * (-k - hv * dkdqy);
    if (a.wantZb) {
      acc_add_from(&a.accF[(size_t)n + j], src.acc(1, &a.accF[(size_t)n + j]), beta, mj1 * m.gf * L.s.xi);
      acc_add_from(&a.accF[(size_t)2 * n + j], src.acc(2, &a.accF[(size_t)2 * n + j]), beta, mj2 * m.gf * L.s.xi);
    }
    }
  }
  if constexpr (FOLD) {   // a dry cell's boundary faces (the face loop above runs for wet cells)
    if (L.s.dry) {
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        const int32_t nb = slot_nb(src.slot(k));
        if (nb < 0 && nb != kNoFace) bnd |= 1u << k;
      }
    }
  }
  if (FOLD && bnd != 0u) {   // boundary faces: c = w . J, the terms k_vjp_bnd_f32 + k_vjp_combine_f32 give
    float gzbB = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!(bnd & (1u << k))) continue;
      const float4 sl = src.slot(k);
      const int32_t bf = boundary_index(slot_nb(sl));
      const float w0 = -sl.z * mj0 / Aj, w1 = -sl.z * mj1 / Aj, w2 = -sl.z * mj2 / Aj;
      float J[24];
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const float4 v = __ldg(&a.bndJ[(size_t)bf * 6 + q]);
        J[4 * q] = v.x; J[4 * q + 1] = v.y; J[4 * q + 2] = v.z; J[4 * q + 3] = v.w;
      }
      g0 += w0 * J[0] + w1 * J[7] + w2 * J[14];
      g1 += w0 * J[1] + w1 * J[8] + w2 * J[15];
      g2 += w0 * J[2] + w1 * J[9] + w2 * J[16];
      gn += w0 * J[3] + w1 * J[10] + w2 * J[17];
      gzbB += w0 * J[4] + w1 * J[11] + w2 * J[18];
      const int32_t info = __ldg(&m.bfInfo[bf]);
      if ((info & 3) == kBcInletQ && !L.s.dry) {
        // total_A = sum L^(5/3) h / n over the group's wet cells (bc_2D.jl:673-676)
        const double gTA = grpTA[info >> 2], lp = m.bfLp53[bf], nm = cp.w;
        g0 += (float)(gTA * lp / nm);
        gn += (float)(gTA * (-lp * (double)L.s.h / (nm * nm)));
      }
    }
    if (a.wantZb && gzbB != 0.0f) acc_add(&a.accF[(size_t)3 * n + j], beta, gzbB);
  }
  if (a.resChain) {   // n = f(state): dL/dn into the state and the function's parameters
    if (gn != 0.0f) {
      const ResJac<float> J =
          manning_jac<float>(m.res, L.s.h, L.s.hu, L.s.hv, m.res.ks ? (float)m.res.ks[j] : 0.0f, L.s.dry);
      g0 += gn * J.dh;
      g1 += gn * J.dqx;
      g2 += gn * J.dqy;
#pragma unroll
      for (int k = 0; k < 4; ++k) acc_add(&a.accRes[(size_t)k * n + j], beta, gn * J.dp[k]);
    }
  } else if (a.udeChain) {   // the network's VJP takes it on (dL/dn, or dL/dF of the closure)
    a.udeGn[j] = (double)(beta * gn);
  } else if (a.wantN && gn != 0.0f) {
    acc_add_from(&a.accF[j], src.acc(0, &a.accF[j]), beta, gn);
  }
  const float mask = (L.s.dry && !NOMASK) ? 0.0f : 1.0f;
  const float e0 = src.extra_own(0), e1 = src.extra_own(1), e2 = src.extra_own(2);
  out[j] = mask * (cSelf * mj0 + cExtra * e0 + beta * g0);
  out[n + j] = mask * (cSelf * mj1 + cExtra * e1 + beta * g1);
  out[2 * n + j] = mask * (cSelf * mj2 + cExtra * e2 + beta * g2);
}

// The interior VJP runs as the programmatic dependent of the boundary VJP
// (hg_pdl.cuh): the boundary kernel waits for the kernels before it and then
// releases the interior one, whose CTAs fill the SMs beside the boundary
// blocks already resident; the interior waits for the boundary grid only
// before it exits (it reads nothing the boundary kernel writes), so the
// kernels after it see both.

template <int NS, bool NOMASK = false>
__global__ void __launch_bounds__(kBlock, vjp_min_blocks<NS>()) k_vjp_f32(DevMesh m, AdjDev a, StateF32 Q, const float* __restrict__ mu,
                                                    const float* __restrict__ extra, float* out, float cSelf,
                                                    float cExtra, float beta) {
  pdl_release_dependents();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m.n) vjp_cell<NS, false, GlobalSrc, NOMASK>(m, a, j, GlobalSrc{m, Q, mu, extra, j}, out, cSelf, cExtra, beta);
  pdl_wait_prerequisites();
}

// Pipelined persistent VJP (the stage kernel's k_stage_pipe_f32 scheme): each
// CTA walks 256-cell tiles; while it computes one, cp.async copies bring the
// next tile's slot records (DevMesh::SLp, tile-local neighbours), state,
// parameter, source and cotangent records and its halo's (DevMesh::halo)
// into the other of two shared-memory buffers.  The arithmetic is vjp_cell's.
constexpr int kVTile = kStageBlockF32;
template <int NS>
struct VjpTile {
  static constexpr uint32_t kRec = kVTile * sizeof(float4), kF = kVTile * sizeof(float);
  static constexpr uint32_t kH16 = kHaloMax * sizeof(float4), kH4 = kHaloMax * sizeof(float);
  static constexpr uint32_t kSL = 0, kX = NS * kRec, kCP = kX + kRec, kCS = kCP + kRec;
  static constexpr uint32_t kMU = kCS + kRec, kEX = kMU + 3 * kF;
  static constexpr uint32_t kHX = kEX + 3 * kF, kHP = kHX + kH16, kHA = kHP + kH16, kHM = kHA + kH4;
  static constexpr uint32_t kACC = (kHM + 3 * kH4 + 15u) & ~15u;   // the own cells' accumulators (acc_prefetched)
  static constexpr uint32_t kBuf = (kACC + 3 * kVTile * (uint32_t)sizeof(float2) + 127u) & ~127u;
  static constexpr uint32_t kSmem = 2 * kBuf;
};
template <int NS>
struct TileSrc {
  const unsigned char* B;
  int tid;
  bool hasExtra;   // no cotangent carried in: the extra slab is not filled
  int base;                  // the tile's first cell
  const int32_t* haloIds;    // the tile's halo cell ids (DevMesh::halo)
  const AdjDev* ad;          // which accumulators the tile holds (acc_prefetched)
  __device__ const float4* rec(uint32_t off) const { return reinterpret_cast<const float4*>(B + off); }
  __device__ const float* flt(uint32_t off) const { return reinterpret_cast<const float*>(B + off); }
  __device__ float4 x() const { return rec(VjpTile<NS>::kX)[tid]; }
  __device__ float4 cp() const { return rec(VjpTile<NS>::kCP)[tid]; }
  __device__ float4 cs() const { return rec(VjpTile<NS>::kCS)[tid]; }
  __device__ float mu_own(int b) const { return flt(VjpTile<NS>::kMU)[b * kVTile + tid]; }
  __device__ float extra_own(int b) const { return hasExtra ? flt(VjpTile<NS>::kEX)[b * kVTile + tid] : 0.0f; }
  __device__ float4 slot(int k) const { return rec(VjpTile<NS>::kSL)[k * kVTile + tid]; }
  __device__ VjpNbr nbr(int nb) const {
    const int li = nb & 511;
    if (li < kVTile)
      return VjpNbr{rec(VjpTile<NS>::kX)[li], rec(VjpTile<NS>::kCP)[li], rec(VjpTile<NS>::kCS)[li].z,
                    flt(VjpTile<NS>::kMU)[li], flt(VjpTile<NS>::kMU)[kVTile + li],
                    flt(VjpTile<NS>::kMU)[2 * kVTile + li]};
    const int h = li - kVTile;
    return VjpNbr{rec(VjpTile<NS>::kHX)[h], rec(VjpTile<NS>::kHP)[h], flt(VjpTile<NS>::kHA)[h],
                  flt(VjpTile<NS>::kHM)[h], flt(VjpTile<NS>::kHM)[kHaloMax + h],
                  flt(VjpTile<NS>::kHM)[2 * kHaloMax + h]};
  }
  __device__ int cell(int nb) const {   // the neighbour's cell id
    const int li = nb & 511;
    return li < kVTile ? base + li : __ldg(&haloIds[li - kVTile]);
  }
  __device__ float2 acc(int q, const float2* p) const {
    return acc_prefetched(*ad, q) ? reinterpret_cast<const float2*>(B + VjpTile<NS>::kACC)[q * kVTile + tid] : *p;
  }
};

// A tile's copies in two parts: the records that stay fixed during the
// reverse sweep (mesh records, the stage state), and the cotangents, which
// the kernel before this one writes.
template <int NS>
__device__ __forceinline__ void vjp_issue_fixed(const DevMesh& m, StateF32 Q, int t, unsigned char* B, int hid) {
  using T = VjpTile<NS>;
  const int tid = threadIdx.x, n = m.n;
  const int c = t * kVTile + tid;
  if (c < n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) cp_async16(B + T::kSL + (k * kVTile + tid) * 16, &m.SLp[(size_t)k * n + c]);
    cp_async16(B + T::kX + tid * 16, &Q.x[c]);
    cp_async16(B + T::kCP + tid * 16, &m.CP[c]);
    cp_async16(B + T::kCS + tid * 16, &m.CS[c]);
  }
  if (hid >= 0) {
    cp_async16(B + T::kHX + tid * 16, &Q.x[hid]);
    cp_async16(B + T::kHP + tid * 16, &m.CP[hid]);
    cp_async4(B + T::kHA + tid * 4, &m.CS[hid].z);
  }
}
template <int NS>
__device__ __forceinline__ void vjp_issue_cot(const DevMesh& m, const AdjDev& a, const float* mu, const float* extra,
                                              int t, unsigned char* B, int hid) {
  using T = VjpTile<NS>;
  const int tid = threadIdx.x, n = m.n;
  const int c = t * kVTile + tid;
  if (c < n) {
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      cp_async4(B + T::kMU + (b * kVTile + tid) * 4, &mu[(size_t)b * n + c]);
      if (extra) cp_async4(B + T::kEX + (b * kVTile + tid) * 4, &extra[(size_t)b * n + c]);
      // the accumulators, which the kernel before this one may have updated
      if (acc_prefetched(a, b)) cp_async8(B + T::kACC + (b * kVTile + tid) * 8, &a.accF[(size_t)b * n + c]);
    }
  }
  if (hid >= 0) {
#pragma unroll
    for (int b = 0; b < 3; ++b) cp_async4(B + T::kHM + (b * kHaloMax + tid) * 4, &mu[(size_t)b * n + hid]);
  }
}
template <int NS>
__device__ __forceinline__ void vjp_issue(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu,
                                          const float* extra, int t, unsigned char* B, int hid) {
  vjp_issue_fixed<NS>(m, Q, t, B, hid);
  vjp_issue_cot<NS>(m, a, mu, extra, t, B, hid);
}

// The inlet groups' total_A and Q cotangents of the folded boundary VJP: for
// each group of the tile's mask gm, the whole CTA strides over the group's
// faces, then a fixed reduction (shuffle tree per warp, the warps' sums in
// order).  Every CTA that needs a group's total_A cotangent forms it; the CTA
// of tile grpTile[g] alone adds the Q cotangent.  sRed: 2 x (warps) doubles.
__device__ void fold_group_sums(const DevMesh& m, const AdjDev& a, const float* __restrict__ mu, uint32_t gm, int t,
                                double betaD, double* sGrp, double* sRed) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5, n = m.n;
  for (int g = 0; g < m.nInlet; ++g) {
    if (!((gm >> g) & 1u)) continue;
    double sTA = 0.0, sQ = 0.0;
    constexpr int U = 4;   // faces per thread in flight at once
    const int e1 = m.inletOff[g + 1];
    for (int e0 = m.inletOff[g] + threadIdx.x; e0 < e1; e0 += U * blockDim.x) {
      float4 iw[U], J1[U], J3[U], J4[U], J5[U];
      float m0[U], m1[U], m2[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + u * blockDim.x;
        iw[u] = e < e1 ? __ldg(&a.inletW[e]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int bf = __float_as_int(iw[u].x), j = __float_as_int(iw[u].y);   // 0, 0 past the end: weight 0
        const float4* Jp = a.bndJ + (size_t)bf * 6;
        J1[u] = __ldg(Jp + 1); J3[u] = __ldg(Jp + 3); J4[u] = __ldg(Jp + 4); J5[u] = __ldg(Jp + 5);
        m0[u] = mu[j]; m1[u] = mu[n + j]; m2[u] = mu[2 * n + j];
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float w0 = -iw[u].z * m0[u], w1 = -iw[u].z * m1[u], w2 = -iw[u].z * m2[u];
        // J[5], J[6] | J[12], J[13] | J[19], J[20]
        sQ += (double)(w0 * J1[u].y + w1 * J3[u].x + w2 * J4[u].w);
        sTA += (double)(w0 * J1[u].z + w1 * J3[u].y + w2 * J5[u].x);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      sTA += __shfl_xor_sync(0xffffffffu, sTA, o);
      sQ += __shfl_xor_sync(0xffffffffu, sQ, o);
    }
    if (lane == 0) {
      sRed[w] = sTA;
      sRed[nw + w] = sQ;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0.0, q = 0.0;
      for (int k = 0; k < nw; ++k) {
        ta += sRed[k];
        q += sRed[nw + k];
      }
      sGrp[g] = ta;
      if (a.grpTile[g] == t) a.gQ[g] += betaD * q;
    }
    __syncthreads();
  }
}

// Tiles 0..G-1 go to the G CTAs in order, the rest to whichever CTA asks next
// (a.tileTicket[0]): a CTA that starts late -- its SM still busy with the
// boundary VJP beside it, or still waiting on the kernel before it -- takes
// fewer tiles instead of finishing late (with the boundary faces folded in,
// static tiles b, b + G, ... measured 7 % slower per forward+adjoint step).
// Each cell is still computed by one thread with the same arithmetic, so the
// result does not depend on the assignment.
// FOLD: launched as the programmatic dependent of the kernel before it, which
// it waits for after the first tile's fixed records are in flight (and
// before anything that kernel writes: cotangents, accumulators, the tile
// tickets its last CTA resets).  MINB: CTAs per SM the registers allow.
template <int NS, bool FOLD, int MINB = 2>
__global__ void __launch_bounds__(kVTile, MINB) k_vjp_pipe_f32(DevMesh m, AdjDev a, StateF32 Q, const float* mu,
                                                           const float* extra, float* out, float cSelf, float cExtra,
                                                           float beta, double betaD) {
  using T = VjpTile<NS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int sNext[2];   // alternate slots: a slot is rewritten two barriers after its last read
  __shared__ double sGrp[kFoldMaxGroups];   // FOLD: the tile's inlet groups' total_A cotangents
  __shared__ double sRed[2 * (kVTile / 32)];
  const int n = m.n, nTiles = (n + kVTile - 1) / kVTile, tid = threadIdx.x, G = gridDim.x;
  auto halo_id = [&](int t) { return (t < nTiles && tid < kHaloMax) ? m.halo[(size_t)t * kHaloMax + tid] : -1; };
  auto take = [&] { return G + (int)atomicAdd(&a.tileTicket[0], 1u); };
  // Tickets are taken two tiles ahead (thread 0 holds the one after next in
  // `ahead`), so an atomic's round trip overlaps a tile's arithmetic.
  pdl_release_dependents();
  int t = blockIdx.x;   // < nTiles: the grid is at most the tile count
  int ahead = 0;
  if constexpr (FOLD) {
    vjp_issue_fixed<NS>(m, Q, t, smem, halo_id(t));
    pdl_wait_prerequisites();
    vjp_issue_cot<NS>(m, a, mu, extra, t, smem, halo_id(t));
  } else {
    vjp_issue<NS>(m, a, Q, mu, extra, t, smem, halo_id(t));
  }
  if (tid == 0) {
    sNext[0] = take();
    ahead = take();
  }
  cp_async_commit();
  __syncthreads();
  int tn = sNext[0];
  int hidNext = halo_id(tn);
  int b = 0, slot = 1;
  while (t < nTiles) {
    if (tn < nTiles) vjp_issue<NS>(m, a, Q, mu, extra, tn, smem + (b ^ 1) * T::kBuf, hidNext);
    cp_async_commit();
    if (tid == 0) sNext[slot] = ahead;
    cp_async_wait<1>();
    __syncthreads();
    const int tnn = sNext[slot];
    if (tid == 0) ahead = take();
    hidNext = halo_id(tnn);
    if constexpr (FOLD) {
      const uint32_t gm = m.nInlet > 0 ? __ldg(&a.tileGrp[t]) : 0u;   // the same for the whole CTA
      if (gm) fold_group_sums(m, a, mu, gm, t, betaD, sGrp, sRed);   // ends with a barrier
    }
    const int j = t * kVTile + tid;
    if (j < n)
      vjp_cell<NS, FOLD>(m, a, j,
                         TileSrc<NS>{smem + b * T::kBuf, tid, extra != nullptr, t * kVTile,
                                     m.halo + (size_t)t * kHaloMax, &a},
                         out, cSelf, cExtra, beta, sGrp);
    __syncthreads();   // buffer b is refilled at the top of the next iteration
    if constexpr (FOLD) {   // the step's probe seeds, after the tile's own cotangents
      if (a.probeSeed)
        for (int e = a.tileProbeOff[t] + tid; e < a.tileProbeOff[t + 1]; e += kVTile) {
          const int u = a.tileProbeU[e];
          out[a.probeCell[u]] += a.probeSeed[u];
        }
    }
    t = tn;
    tn = tnn;
    b ^= 1;
    slot ^= 1;
  }
  cp_async_wait<0>();
  if (tid == 0) {
    __threadfence();   // this CTA's takes come before its finish count
    if (atomicAdd(&a.tileTicket[1], 1u) == (unsigned)G - 1) {   // the last CTA out: every take is done
      atomicExch(&a.tileTicket[0], 0u);
      atomicExch(&a.tileTicket[1], 0u);
    }
  }
  pdl_wait_prerequisites();
}

// Per inlet-Q group (one warp each): grpTA = sum over the group's faces of
// the total_A cotangent, gQ += beta sum of the Q cotangent -- lanes stride
// over the faces, a fixed shuffle tree adds them (deterministic).
__device__ void inlet_group_sums(const DevMesh& m, const AdjDev& a, double betaD) {
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int g = threadIdx.x >> 5; g < m.nInlet; g += nw) {
    double sTA = 0.0, sQ = 0.0;
    for (int e = m.inletOff[g] + lane; e < m.inletOff[g + 1]; e += 32) {
      const int bf = a.inletBf[e];
      sTA += __ldcg(&a.bfGradTA[bf]);
      sQ += __ldcg(&a.bfGradQ[bf]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sTA += __shfl_xor_sync(0xffffffffu, sTA, o);
      sQ += __shfl_xor_sync(0xffffffffu, sQ, o);
    }
    if (lane == 0) {
      a.grpTA[g] = sTA;
      a.gQ[g] += betaD * sQ;
    }
  }
}

// Boundary faces of the cells that have any (one thread per such cell; runs
// beside the interior VJP, which reads none of what it writes): ghost-state
// duals in the own state, n, zb, Q and total_A.  Leaves the cell's terms in
// bndG and the Q / total_A cotangents per boundary face; the last block to
// finish sums the latter per inlet group.
template <int NS>
__global__ void __launch_bounds__(64) k_vjp_bnd_f32(DevMesh m, AdjDev a, StateF32 Q, const float* __restrict__ mu,
                                                    double betaD) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.nBndCells) {
    const int j = a.bndCells[i];
    const int n = m.n;
    const float4 cp = __ldg(&m.CP[j]);
    const SideF32 L = make_side_f32(__ldg(&Q.x[j]), cp, m.hsmf, m.hsmLo);
    const float Aj = __ldg(&m.CS[j]).z;
    const float mj0 = mu[j], mj1 = mu[n + j], mj2 = mu[2 * n + j];
    float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gn = 0.0f, gzb = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const float4 sl = __ldg(&m.SL[(size_t)k * n + j]);
      const int32_t nb = slot_nb(sl);
      if (nb >= 0 || nb == kNoFace) continue;
      const float nx = sl.x, ny = sl.y, len = sl.z;
      const int32_t bf = boundary_index(nb);
      const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
      const float w0 = -len * mj0 / Aj, w1 = -len * mj1 / Aj, w2 = -len * mj2 / Aj;
      const Side<F7> L7 = seeded<F7>(L.s, 4);
      const F7 man = F7::seed(cp.w, 3);
      const F7 qin = F7::seed(type == kBcInletQ ? (float)m.inletQ[grp] : 0.0f, 5);
      const F7 ta = F7::seed(type == kBcInletQ ? (float)m.totalA[grp] : 1.0f, 6);
      const Side<F7> R7 = ghost_state<F7>(L7, type, F7(nx), F7(ny), F7(m.hsmf),
                                          F7(type == kBcExitH ? (float)m.exitWse[grp] : 0.0f), qin, ta,
                                          F7(m.bfLp23f[bf]), man);
      F7 ex(L.excess);
      if (L.s.dry) ex.d[0] = -1.0f;   // excess = h_small - (xi + hstill) for a dry cell
      F7 dxi = (R7.h - L7.h) + ex;
      if (type == kBcExitH && !R7.dry) dxi.v = m.bfExitRel[bf] - (L.s.xi + L.xlo);   // as the forward pass
      int bank = -1;   // the forward pass's wall test (bank_wall_f64)
      if (type == kBcExitH && L.s.dry != R7.dry)
        bank = L.s.dry ? bank_exit_f64(m, grp, j) : bank_wall_f64(m, L.s.xi, L.xlo, j, j);
      F7 F[3];
      riemann_flux<F7>(m.riemann, L7, R7, dxi, F7(m.gf), F7(nx), F7(ny), F7(m.hsmf), F, bank);
      float c[7];
#pragma unroll
      for (int d = 0; d < 7; ++d) c[d] = w0 * F[0].d[d] + w1 * F[1].d[d] + w2 * F[2].d[d];
      g0 += c[0]; g1 += c[1]; g2 += c[2];
      gn += c[3];
      gzb += c[4];
      a.bfGradQ[bf] = (double)c[5];
      a.bfGradTA[bf] = (double)c[6];
    }
    float* o = a.bndG + (size_t)5 * i;
    o[0] = g0; o[1] = g1; o[2] = g2; o[3] = gn; o[4] = gzb;
  }
  if (m.nInlet > 0) {
    __shared__ bool last;
    __threadfence();   // this block's face cotangents before its finish count
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&a.tileTicket[2], 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) {
      __threadfence();
      inlet_group_sums(m, a, betaD);
      if (threadIdx.x == 0) a.tileTicket[2] = 0u;
    }
  }
}

// Folded boundary VJP: the flux Jacobian of boundary face bf at state s of a
// segment (records X + s n, inlet totals tot + s totStride), by the
// 7-direction duals k_vjp_bnd_f32 takes, without the cotangent.
__global__ void __launch_bounds__(128) k_bnd_jac_f32(DevMesh m, AdjDev a, const float4* __restrict__ X, int nStates,
                                                     const double* __restrict__ tot, size_t totStride, float4* J) {
  const int nbf = m.nbf, n = m.n;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nStates * nbf) return;
  const int s = (int)(t / nbf), bf = (int)(t - (int64_t)s * nbf);
  const int2 cs = a.bfSlot[bf];
  const int j = cs.x;
  const float4 sl = __ldg(&m.SL[(size_t)cs.y * n + j]);
  const float4 cp = __ldg(&m.CP[j]);
  const SideF32 L = make_side_f32(__ldg(&X[(size_t)s * n + j]), cp, m.hsmf, m.hsmLo);
  const float nx = sl.x, ny = sl.y;
  const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
  const Side<F7> L7 = seeded<F7>(L.s, 4);
  const F7 man = F7::seed(cp.w, 3);
  const F7 qin = F7::seed(type == kBcInletQ ? (float)m.inletQ[grp] : 0.0f, 5);
  const F7 ta = F7::seed(type == kBcInletQ ? (float)tot[(size_t)s * totStride + grp] : 1.0f, 6);
  const Side<F7> R7 = ghost_state<F7>(L7, type, F7(nx), F7(ny), F7(m.hsmf),
                                      F7(type == kBcExitH ? (float)m.exitWse[grp] : 0.0f), qin, ta,
                                      F7(m.bfLp23f[bf]), man);
  F7 ex(L.excess);
  if (L.s.dry) ex.d[0] = -1.0f;   // excess = h_small - (xi + hstill) for a dry cell
  F7 dxi = (R7.h - L7.h) + ex;
  if (type == kBcExitH && !R7.dry) dxi.v = m.bfExitRel[bf] - (L.s.xi + L.xlo);   // as the forward pass
  int bank = -1;   // the forward pass's wall test (bank_wall_f64)
  if (type == kBcExitH && L.s.dry != R7.dry)
    bank = L.s.dry ? bank_exit_f64(m, grp, j) : bank_wall_f64(m, L.s.xi, L.xlo, j, j);
  F7 F[3];
  riemann_flux<F7>(m.riemann, L7, R7, dxi, F7(m.gf), F7(nx), F7(ny), F7(m.hsmf), F, bank);
  float v[24];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int d = 0; d < 7; ++d) v[7 * r + d] = F[r].d[d];
  v[21] = v[22] = v[23] = 0.0f;
  float4* o = J + ((size_t)s * nbf + bf) * 6;
#pragma unroll
  for (int q = 0; q < 6; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// After both VJP kernels: each boundary cell's terms into out (when wet) and
// the n / zb accumulators, then its inlet total_A terms (bc_2D.jl:673-676:
// total_A = sum L^(5/3) h / n over the group's wet cells) into out and gN.
__device__ __forceinline__ double depth_f64(const DevMesh& m, StateF32 Q, int c) {
  const float4 x = Q.x[c];
  const float4 cp = m.CP[c];
  return ((double)x.x + (double)x.y) + ((double)cp.x + (double)cp.y);
}

// The seed of distinct probe cell u: mu_xi[c] += sum over the probes at c (in
// probe order) of scale 2 (h - obs_p), when c is wet (mask; otherwise in any
// case: a state no clamp follows, as Tsit5's).
__device__ __forceinline__ void probe_seed(const DevMesh& m, StateF32 Q, float* mu, const ProbeCsr& pc,
                                           const double* __restrict__ obs, double scale, int u, bool mask) {
  const int c = pc.cell[u];
  const float4 cp = m.CP[c];
  const SideF32 L = make_side_f32(Q.x[c], cp, m.hsmf, m.hsmLo);
  if (mask && L.s.dry) return;
  const double h = depth_f64(m, Q, c);
  double acc = 0.0;
  for (int i = pc.off[u]; i < pc.off[u + 1]; ++i) acc += scale * 2.0 * (h - obs[pc.idx[i]]);
  mu[c] += (float)acc;
}

// The probe terms of a state Q of the run, by one whole block: its loss sum
// over the probes p of (h - obs_p)^2 into a.loss (a fixed-order reduction) and
// the seeds of the probe cells (skipBnd: not those that are boundary cells,
// whose seed the combine adds after its own terms).
__device__ __forceinline__ void probe_block(const DevMesh& m, const AdjDev& a, StateF32 Q, float* mu,
                                            const ProbeCsr& pc, const int32_t* __restrict__ probes,
                                            const double* __restrict__ obs, int np, double scale, bool skipBnd) {
  for (int u = threadIdx.x; u < pc.nCells; u += blockDim.x)
    if (!skipBnd || !pc.isBnd[u]) probe_seed(m, Q, mu, pc, obs, scale, u, !a.noMask);
  double s = 0.0;
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    const double e = depth_f64(m, Q, probes[p]) - obs[p];
    s += e * e;
  }
  const double t = block_sum(s);
  if (threadIdx.x == 0) a.loss[0] += t;
}

// In the reverse sweep, with no combine to join: the probe terms of the state.
__global__ void __launch_bounds__(256) k_probe_f32(DevMesh m, AdjDev a, StateF32 Q, float* mu, ProbeCsr pc,
                                                   const int32_t* __restrict__ probes,
                                                   const double* __restrict__ obs, int np, double scale) {
  pdl_enter();
  probe_block(m, a, Q, mu, pc, probes, obs, np, scale, false);
}

// Folded reverse sweep: the probe terms of a segment's states, one block per
// step s (the state after step s - 1): each distinct probe cell's seed (as
// probe_seed adds it; 0 for a dry cell) and the loss sum (probe_block's order).
__global__ void __launch_bounds__(256) k_probe_seg_f32(DevMesh m, const float4* __restrict__ X, int s0, int sFirst,
                                                       ProbeCsr pc, const int32_t* __restrict__ probes,
                                                       const double* __restrict__ obs, int np, double scale,
                                                       float* seeds, double* lossPart) {
  const int s = sFirst + blockIdx.x;
  const StateF32 Q{const_cast<float4*>(X) + (size_t)(s - s0) * m.n, nullptr};
  const double* ob = obs + (size_t)(s - 1) * np;
  for (int u = threadIdx.x; u < pc.nCells; u += blockDim.x) {
    const int c = pc.cell[u];
    const SideF32 L = make_side_f32(Q.x[c], m.CP[c], m.hsmf, m.hsmLo);
    double acc = 0.0;
    if (!L.s.dry) {
      const double h = depth_f64(m, Q, c);
      for (int i = pc.off[u]; i < pc.off[u + 1]; ++i) acc += scale * 2.0 * (h - ob[pc.idx[i]]);
    }
    seeds[(size_t)blockIdx.x * pc.nCells + u] = (float)acc;
  }
  double sum = 0.0;
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    const double e = depth_f64(m, Q, probes[p]) - ob[p];
    sum += e * e;
  }
  const double t = block_sum(sum);
  if (threadIdx.x == 0) lossPart[s - 1] = t;
}

__global__ void k_loss_parts(AdjDev a, const double* __restrict__ lossPart, int sLast) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double l = a.loss[0];
  for (int s = sLast; s >= 1; --s) l += lossPart[s - 1];
  a.loss[0] = l;
}

// 256-thread blocks: the probe block reduces the loss in the order of the
// standalone k_probe_f32.
constexpr int kCombineBlock = 256;
// pj.np > 0 (the stage-1 VJP of a step with probes): the last block does the
// probe terms of the VJP's state (the seeds of probe cells that are not
// boundary cells, and the loss), and each boundary cell that is a probe cell
// adds its seed after its own terms -- the order of two separate kernels.
__global__ void __launch_bounds__(kCombineBlock) k_vjp_combine_f32(DevMesh m, AdjDev a, StateF32 Q, float* out,
                                                                   float beta, double betaD, ProbeJob pj) {
  pdl_enter();
  if (pj.np > 0 && blockIdx.x == gridDim.x - 1) {
    probe_block(m, a, Q, out, pj.pc, pj.probes, pj.obs, pj.np, pj.scale, true);
    return;
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nBndCells) return;
  const int j = a.bndCells[i];
  const int n = m.n;
  const float4 cp = m.CP[j];
  const SideF32 L = make_side_f32(Q.x[j], cp, m.hsmf, m.hsmLo);
  const float* g = a.bndG + (size_t)5 * i;
  const bool chainN = a.resChain || a.udeChain == 1;   // dL/dn of the cell goes to n's function
  if (a.wantN && !chainN && g[3] != 0.0f) acc_add(&a.accF[j], beta, g[3]);
  if (a.wantZb && g[4] != 0.0f) acc_add(&a.accF[(size_t)3 * n + j], beta, g[4]);
  if (L.s.dry && !a.noMask) return;
  // n = f(state): the boundary faces' and the inlet conveyance's dL/dn of the
  // cell into its state and the function's parameters
  double gnRes = chainN ? (double)g[3] : 0.0;
  out[j] += beta * g[0];
  out[n + j] += beta * g[1];
  out[2 * n + j] += beta * g[2];
  // (total_A sums the wet cells only: a dry cell's state does not enter it)
  for (int p = L.s.dry ? a.bndInOff[i + 1] : a.bndInOff[i]; p < a.bndInOff[i + 1]; ++p) {
    const double gTA = a.grpTA[a.bndInGrp[p]];
    const double coef = a.bndInCoef[p], nm = cp.w;
    out[j] += (float)(betaD * gTA * coef / nm);
    const double gnc = gTA * (-coef * (double)L.s.h / (nm * nm));
    if (chainN) gnRes += gnc;
    else if (a.wantN) a.gN[j] += betaD * gnc;
  }
  if (a.udeChain == 1 && gnRes != 0.0) a.udeGn[j] += betaD * gnRes;
  if (a.resChain && gnRes != 0.0) {
    const ResJac<double> J = manning_jac<double>(m.res, (double)L.s.h, (double)L.s.hu, (double)L.s.hv,
                                                 m.res.ks ? m.res.ks[j] : 0.0, L.s.dry);
    out[j] += (float)(betaD * gnRes * J.dh);
    out[n + j] += (float)(betaD * gnRes * J.dqx);
    out[2 * n + j] += (float)(betaD * gnRes * J.dqy);
    for (int k = 0; k < 4; ++k) a.gResP[(size_t)k * n + j] += betaD * gnRes * J.dp[k];
  }
  if (pj.np > 0 && a.bndProbe[i] >= 0) probe_seed(m, Q, out, pj.pc, pj.obs, pj.scale, a.bndProbe[i], !a.noMask);
}

__global__ void k_fold_accumulators_f32(DevMesh m, AdjDev a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m.n) return;
  double* dst[4] = {a.gN, a.gS0x, a.gS0y, a.gZb};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 v = a.accF[(size_t)k * m.n + j];
    dst[k][j] += (double)v.x + (double)v.y;
  }
  if (a.resChain) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 v = a.accRes[(size_t)k * m.n + j];
      a.gResP[(size_t)k * m.n + j] += (double)v.x + (double)v.y;
    }
  }
}

}  // namespace

namespace {
// The interior VJP takes the pipelined persistent kernel wherever it can run
// (degree <= 4, the tile tables built, 16-byte aligned state records) -- a
// fixed choice, so runs reproduce; HG_VJP_KERNEL=gather forces the
// block-per-128-cells kernel.
bool vjp_gather_forced() {
  static const bool on = [] {
    const char* e = std::getenv("HG_VJP_KERNEL");
    return e && std::strcmp(e, "gather") == 0;
  }();
  return on;
}

bool pipe_usable(const DevMesh& m, StateF32 Q) {
  auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  return m.nslot <= 4 && !vjp_gather_forced() && m.SLp && m.halo && a16(m.SLp) && a16(m.CP) && a16(m.CS) &&
         a16(Q.x);
}

// The pipelined persistent interior VJP (a grid of the CTAs resident at once).
template <int NS, bool FOLD, int MINB = 2>
void launch_vjp_pipe(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra, float* out,
                     float cSelf, float cExtra, float beta, double betaD, bool pdl, cudaStream_t st) {
  using T = VjpTile<NS>;
  static const int grid = [] {
    cudaFuncSetAttribute(k_vjp_pipe_f32<NS, FOLD, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)T::kSmem);
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_vjp_pipe_f32<NS, FOLD, MINB>, kVTile, T::kSmem) !=
            cudaSuccess ||
        per < 1)
      per = 1;
    return (sms > 0 ? sms : 1) * per;
  }();
  const int tiles = (m.n + kVTile - 1) / kVTile;
  launch_k(pdl, k_vjp_pipe_f32<NS, FOLD, MINB>, tiles < grid ? tiles : grid, kVTile, T::kSmem, st, m, a, Q, mu,
           extra, out, cSelf, cExtra, beta, betaD);
}

// CTAs per SM of the folded interior VJP: 2 (128 registers), or 3 with
// HG_VJP_MINB=3 (80 registers, some spilled); read once per process.
int vjp_fold_minb() {
  static const int v = [] {
    const char* e = std::getenv("HG_VJP_MINB");
    return (e && std::strcmp(e, "3") == 0) ? 3 : 2;
  }();
  return v;
}

// pdl: launched as the programmatic dependent of the boundary VJP just before it.
template <int NS>
void launch_vjp_interior(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra,
                         float* out, float cSelf, float cExtra, float beta, bool pdl, cudaStream_t st) {
  if (a.noMask) {   // the RHS VJP of Tsit5 stages: the gather kernel's unmasked instance
    launch_k(pdl, k_vjp_f32<NS, true>, blocks_for(m.n), kBlock, 0, st, m, a, Q, mu, extra, out, cSelf, cExtra, beta);
    return;
  }
  if constexpr (NS <= 4) {
    if (pipe_usable(m, Q)) {
      launch_vjp_pipe<NS, false>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, (double)beta, pdl, st);
      return;
    }
  }
  launch_k(pdl, k_vjp_f32<NS>, blocks_for(m.n), kBlock, 0, st, m, a, Q, mu, extra, out, cSelf, cExtra, beta);
}

// The boundary VJP, then the interior VJP as its programmatic dependent (both
// on the context's stream, running side by side), then the combine.
template <int NS>
int launch_vjp_ns(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra, float* out,
                  float cSelf, float cExtra, double betaD, cudaStream_t st, const ProbeJob* pj) {
  const float beta = (float)betaD;
  const int nbb = (a.nBndCells + 63) / 64;
  const bool probes = pj && pj->np > 0;
  if (nbb) launch_k(true, k_vjp_bnd_f32<NS>, nbb, 64, 0, st, m, a, Q, mu, betaD);
  launch_vjp_interior<NS>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, nbb > 0, st);
  if (!nbb) {
    if (probes)
      launch_k(true, k_probe_f32, 1, 256, 0, st, m, a, Q, out, pj->pc, pj->probes, pj->obs, pj->np, pj->scale);
    return probes ? 2 : 1;
  }
  const ProbeJob none;
  launch_k(true, k_vjp_combine_f32, (a.nBndCells + kCombineBlock - 1) / kCombineBlock + (probes ? 1 : 0), kCombineBlock,
           0, st, m, a, Q, out, beta, betaD, probes ? *pj : none);
  return 3;
}
}  // namespace

bool vjp_fold_usable(const DevMesh& m, const AdjDev& a, StateF32 Q) {
  static const bool off = [] {   // HG_VJP_FOLD=0: the separate boundary and combine kernels
    const char* e = std::getenv("HG_VJP_FOLD");
    return e && std::strcmp(e, "0") == 0;
  }();
  return !off && pipe_usable(m, Q) && a.bfSlot && a.tileGrp && a.grpTile && m.nInlet <= kFoldMaxGroups;
}

int launch_bnd_jac_f32(const DevMesh& m, const AdjDev& a, const float4* X, int nStates, const double* tot,
                       size_t totStride, float4* J, cudaStream_t st) {
  const int64_t work = (int64_t)nStates * m.nbf;
  if (work <= 0) return 0;
  k_bnd_jac_f32<<<(unsigned)((work + 127) / 128), 128, 0, st>>>(m, a, X, nStates, tot, totStride, J);
  return 1;
}

int launch_probe_seg_f32(const DevMesh& m, const float4* X, int s0, int sFirst, int nSteps, const ProbeCsr& pc,
                         const int32_t* probes, const double* obs, int32_t np, double scale, float* seeds,
                         double* lossPart, cudaStream_t st) {
  if (nSteps <= 0 || np <= 0) return 0;
  k_probe_seg_f32<<<nSteps, 256, 0, st>>>(m, X, s0, sFirst, pc, probes, obs, np, scale, seeds, lossPart);
  return 1;
}
int launch_loss_parts(const AdjDev& a, const double* lossPart, int sLast, cudaStream_t st) {
  if (sLast < 1) return 0;
  k_loss_parts<<<1, 32, 0, st>>>(a, lossPart, sLast);
  return 1;
}

int launch_vjp_f32_folded(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra,
                          float* out, float cSelf, float cExtra, double betaD, cudaStream_t st, const ProbeJob* pj) {
  const float beta = (float)betaD;
  const bool three = vjp_fold_minb() == 3;
  if (m.nslot <= 3) {
    if (three) launch_vjp_pipe<3, true, 3>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, betaD, true, st);
    else launch_vjp_pipe<3, true, 2>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, betaD, true, st);
  } else {
    if (three) launch_vjp_pipe<4, true, 3>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, betaD, true, st);
    else launch_vjp_pipe<4, true, 2>(m, a, Q, mu, extra, out, cSelf, cExtra, beta, betaD, true, st);
  }
  if (pj && pj->np > 0) {
    launch_k(true, k_probe_f32, 1, 256, 0, st, m, a, Q, out, pj->pc, pj->probes, pj->obs, pj->np, pj->scale);
    return 2;
  }
  return 1;
}

int launch_vjp_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, const float* mu, const float* extra, float* out,
                   float cSelf, float cExtra, double betaD, cudaStream_t st, const ProbeJob* pj) {
  if (m.nslot <= 3) return launch_vjp_ns<3>(m, a, Q, mu, extra, out, cSelf, cExtra, betaD, st, pj);
  if (m.nslot <= 4) return launch_vjp_ns<4>(m, a, Q, mu, extra, out, cSelf, cExtra, betaD, st, pj);
  return launch_vjp_ns<8>(m, a, Q, mu, extra, out, cSelf, cExtra, betaD, st, pj);
}
void launch_probe_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, float* mu, const ProbeCsr& pc,
                      const int32_t* probes, const double* obs, int32_t nprobe, double scale, cudaStream_t st) {
  if (nprobe > 0) launch_k(true, k_probe_f32, 1, 256, 0, st, m, a, Q, mu, pc, probes, obs, nprobe, scale);
}
void launch_fold_accumulators_f32(const DevMesh& m, const AdjDev& a, cudaStream_t st) {
  k_fold_accumulators_f32<<<blocks_for(m.n), kBlock, 0, st>>>(m, a);
}

}  // namespace hg
