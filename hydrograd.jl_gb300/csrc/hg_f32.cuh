// FP32-compensated path: packed cell records, the dry decision from the hi + lo
// pairs, double-float (hi + lo) arithmetic and the wet-wet Roe fast path,
// shared by the forward and adjoint kernels.
//
// Layout (device cell order):
//   X[c]  float4 {xi_hi, xi_lo, qx_hi, qy_hi}   the part of the state a neighbour reads
//   XQ[c] float2 {qx_lo, qy_lo}                 the rest of the compensated state
//   CP[c] float4 {hstill_hi, hstill_lo, zb, n}  per-cell parameters a neighbour reads
//   CS[c] float4 {S0x, S0y, area, 0}            per-cell source data
//   SL[k n + c] float4 {nx, ny, L, nb as bits}  edge slot k of cell c
#pragma once
#include <cstdint>

#include "hg_device.cuh"
#include "hg_state.hpp"

namespace hgd {

struct DepthF32 {
  float h;        // clamped depth
  float excess;   // (h_clamped - hstill) - xi: 0 when wet, the clamp shift when dry
  bool dry;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Depth h = xi + hstill with the reference's dry decision h <= h_small, from
// the hi + lo pairs of xi and hstill and h_small = hsmf + hsmLo, in FP32
// only (GB300 issues FP64 at a small fraction of the FP32 rate):
// xh + hh - hsmf is formed exactly by two error-free sums, the lo terms are
// added to it, and the decision takes a tolerance of 2^-46 |xh| + |hh| -- the
// granularity at which the pairs store a clamped cell's xi (dry_xi), so a
// clamped cell stays dry.  The arithmetic error of the difference is below
// 2^-47 of that magnitude, so the decision is the exact one outside the
// tolerance band.
__device__ __forceinline__ DepthF32 depth_f32(float xh, float xl, float hh, float hl, float hsmf, float hsmLo) {
  DepthF32 d;
  float s, e;
  two_sum(xh, hh, s, e);                 // s + e = xh + hh exactly
  const float low = (e + xl) + hl;
  const float est = s + low;             // depth estimate
  float t, te;
  two_sum(s, -hsmf, t, te);              // t + te = s - hsmf exactly
  const float diff = t + ((te + low) - hsmLo);
  const float mag = fabsf(xh) + fabsf(hh);
  d.dry = diff <= 1.4210854715202004e-14f * mag;
  d.excess = d.dry ? (hsmf - est) : 0.0f;
  d.h = d.dry ? hsmf : est;
  return d;
}

struct SideF32 {
  Side<float> s;
  float xlo;      // lo part of xi
  float excess;   // see DepthF32
};

__device__ __forceinline__ SideF32 make_side_f32(float4 x, float4 p, float hsmf, float hsmLo) {
  SideF32 r;
  const DepthF32 d = depth_f32(x.x, x.y, p.x, p.y, hsmf, hsmLo);
  r.s.xi = x.x;
  r.xlo = x.y;
  r.s.hst = p.x;
  r.s.zb = p.z;
  r.s.dry = d.dry;
  r.s.h = d.h;
  r.s.hu = d.dry ? 0.0f : x.z;
  r.s.hv = d.dry ? 0.0f : x.w;
  r.excess = d.excess;
  return r;
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// (ah + al) + d, renormalised.
__device__ __forceinline__ void df_add(float ah, float al, float d, float& rh, float& rl) {
  float s, e;
  two_sum(ah, d, s, e);
  e += al;
  fast_two_sum(s, e, rh, rl);
}
// (ah + al) + (bh + bl), renormalised.
__device__ __forceinline__ void df_add2(float ah, float al, float bh, float bl, float& rh, float& rl) {
  float s, e;
  two_sum(ah, bh, s, e);
  e += al + bl;
  fast_two_sum(s, e, rh, rl);
}

__device__ __forceinline__ int32_t slot_nb(float4 s) { return __float_as_int(s.w); }

// Quantities of a wet cell that the Roe flux uses on every one of its faces,
// formed once per cell: velocity, sqrt(h), pre-balanced pressure
// p = g/2 (smooth_pow2(xi) + 2 xi hstill) and the advective flux tensor
// [[hu u, hu v], [hv u, hv v]].
struct OwnF32 {
  float u, v, s, p;
  float fxx, fxy, fyx, fyy;
};

// FP32 forms of the smooth_* helpers on the wet path.  smooth_abs(x) =
// sqrt(x^2 + eps) is |x| to FP32 precision once |x| > 1e-4 (eps / x^2 < 2.3e-8
// < 2^-24); sqrt(h + eps) and 1/h of a wet cell (h > h_small) come from one
// reciprocal square root: sqrt(h) = h r, 1/h = r^2 with r = rsqrt(h).
__device__ __forceinline__ float smooth_abs_f32(float x) {
  const float a = fabsf(x);
  return a > 1.0e-4f ? a : sqrtf(fmaf(x, x, eps_c<float>()));
}

__device__ __forceinline__ OwnF32 own_f32(const Side<float>& L, float g) {
  OwnF32 o;
  const float rq = rsqrtf(L.h);
  const float r = rq * rq;
  o.u = L.hu * r;
  o.v = L.hv * r;
  o.s = L.h * rq;
  o.p = 0.5f * g * (smooth_pow2(L.xi) + 2.0f * L.xi * L.hst);
  o.fxx = L.hu * o.u;
  o.fxy = L.hu * o.v;
  o.fyx = L.hv * o.u;
  o.fyy = L.hv * o.v;
  return o;
}

// Well-balancing in FP32.  A cell's RHS is -sum_k F_k L_k / A, and the sum of
// its faces' n_k L_k is zero, so subtracting the own pressure p_L n_k from
// every face's momentum flux leaves the RHS unchanged -- but it removes the
// large own-pressure terms (p ~ g xi hstill) whose sum cancels only to the
// FP32 rounding of the normals and lengths, about 1e-7 of p per cell: in a
// raised pool over a sloping bed that residual drives a spurious flow that
// grows linearly in time.  The wet-wet flux then carries p_R - p_L, formed
// from the exact differences of the hi + lo pairs (pressure_jump_f32); every
// other face subtracts p_L n after the reference solver.
__device__ __forceinline__ float pressure_jump_f32(float g, float xiL, float xiR, float dxi, float hstR,
                                                   float dhst) {
  // (xiR + e)^2 - (xiL + e)^2 + 2 (xiR hstR - xiL hstL)
  //   = dxi (xiR + xiL + 2 e + 2 hstR) + 2 xiL (hstR - hstL)
  return 0.5f * g * (dxi * ((xiR + xiL) + 2.0f * eps_c<float>() + 2.0f * hstR) + 2.0f * xiL * dhst);
}

// Roe flux of a face whose two sides are both wet -- the case in which the
// reference solver (swe_2D_solvers.jl:79-164) takes none of its dry or wall
// branches -- with the own cell's quantities from own_f32, minus p_L n in the
// momentum rows (see pressure_jump_f32; dhst = hstill_R - hstill_L).  The
// algebra is the reference's, regrouped: w1 + w2 = dxi exactly, so
// w1 = dxi/2 + t and w2 = dxi/2 - t with t = (un dxi - nx d1 - ny d2) / (2c),
// and the rows of R |Lambda| w are collected around w1 + w2 and w2 - w1.
__device__ __forceinline__ void roe_flux_wet_f32(const Side<float>& L, const OwnF32& o, const Side<float>& R,
                                                 float dxi, float dhst, float g, float nx, float ny, float F[3]) {
  const float rq = rsqrtf(R.h);
  const float rR = rq * rq;
  const float uR = R.hu * rR, vR = R.hv * rR;
  const float sR = R.h * rq;
  const float rs = 1.0f / (o.s + sR);
  const float uRoe = (o.s * o.u + sR * uR) * rs;
  const float vRoe = (o.s * o.v + sR * vR) * rs;
  const float unRoe = uRoe * nx + vRoe * ny;
  const float gh = g * ((L.h + R.h) * 0.5f);
  const float rc = rsqrtf(gh);
  const float cRoe = gh * rc;   // sqrt(g hRoe)
  const float d1 = R.hu - L.hu, d2 = R.hv - L.hv;
  const float t = (unRoe * dxi - nx * d1 - ny * d2) * (0.5f * rc);
  const float w0 = (ny * d1 - nx * d2 - (uRoe * ny - vRoe * nx) * dxi) * smooth_abs_f32(unRoe);
  const float w1 = (0.5f * dxi + t) * smooth_abs_f32(unRoe - cRoe);
  const float w2 = (0.5f * dxi - t) * smooth_abs_f32(unRoe + cRoe);
  const float sum = w1 + w2, dif = cRoe * (w2 - w1);
  const float A0 = sum;
  const float A1 = ny * w0 + uRoe * sum + nx * dif;
  const float A2 = -nx * w0 + vRoe * sum + ny * dif;
  const float dp = pressure_jump_f32(g, L.xi, R.xi, dxi, R.hst, dhst);   // p_R - p_L
  const float fR1x = R.hu * uR + dp, fR2y = R.hv * vR + dp;
  F[0] = 0.5f * ((L.hu * nx + L.hv * ny) + (R.hu * nx + R.hv * ny) - A0);
  F[1] = 0.5f * ((o.fxx * nx + o.fxy * ny) + (fR1x * nx + R.hu * vR * ny) - A1);
  F[2] = 0.5f * ((o.fyx * nx + o.fyy * ny) + (R.hv * uR * nx + fR2y * ny) - A2);
}

// HLL flux of a face whose two sides are both wet (hll_flux's wet-wet case),
// minus p_L n in the momentum rows as in roe_flux_wet_f32.  With f' a side's
// advective flux and dp = p_R - p_L from the exact differences of the pairs
// (pressure_jump_f32):
//   S_L >= 0:  f'_L;   S_R <= 0:  f'_R + dp n;
//   else       (S_R f'_L - S_L f'_R - S_L dp n + S_L S_R dU) / (S_R - S_L).
__device__ __forceinline__ void hll_flux_wet_f32(const Side<float>& L, const OwnF32& o, const Side<float>& R,
                                                 float dxi, float dhst, float g, float nx, float ny, float F[3]) {
  const float rq = rsqrtf(R.h);
  const float rR = rq * rq;
  const float uR = R.hu * rR, vR = R.hv * rR;
  const float sqR = R.h * rq;
  const float rs = 1.0f / (o.s + sqR);
  const float uRoe = (o.s * o.u + sqR * uR) * rs;
  const float vRoe = (o.s * o.v + sqR * vR) * rs;
  const float unRoe = uRoe * nx + vRoe * ny;
  const float cRoe = sqrtf(g * ((L.h + R.h) * 0.5f));
  const float unL = o.u * nx + o.v * ny, unR = uR * nx + vR * ny;
  const float cL = sqrtf(g * L.h), cR = sqrtf(g * R.h);
  const float sL = fminf(unL - cL, unRoe - cRoe), sR = fmaxf(unR + cR, unRoe + cRoe);
  const float dp = pressure_jump_f32(g, L.xi, R.xi, dxi, R.hst, dhst);
  const float fL0 = L.hu * nx + L.hv * ny;
  const float fL1 = o.fxx * nx + o.fxy * ny;
  const float fL2 = o.fyx * nx + o.fyy * ny;
  const float fR0 = R.hu * nx + R.hv * ny;
  const float fR1 = R.hu * uR * nx + R.hu * vR * ny;
  const float fR2 = R.hv * uR * nx + R.hv * vR * ny;
  if (sL >= 0.0f) {
    F[0] = fL0; F[1] = fL1; F[2] = fL2;
  } else if (sR <= 0.0f) {
    F[0] = fR0; F[1] = fR1 + dp * nx; F[2] = fR2 + dp * ny;
  } else {
    const float r = 1.0f / (sR - sL), sLR = sL * sR;
    F[0] = (sR * fL0 - sL * fR0 + sLR * dxi) * r;
    F[1] = (sR * fL1 - sL * fR1 - sL * dp * nx + sLR * (R.hu - L.hu)) * r;
    F[2] = (sR * fL2 - sL * fR2 - sL * dp * ny + sLR * (R.hv - L.hv)) * r;
  }
}

// ---------------------------------------------------------------------------
// Face-once form (k_stage_face_f32)
// ---------------------------------------------------------------------------
// A face whose two sides are both wet takes the reference solver's wet path
// (swe_2D_solvers.jl:79-164), which is antisymmetric under (a <-> b, n -> -n):
// F(b, a, -n) = -F(a, b, n).  With the own pressure shift of
// pressure_jump_f32 the two cells' terms are then
//   c_a = F(a, b, n) - p_a n,   c_b = F(b, a, -n) + p_b n = -c_a + (p_b - p_a) n,
// so the flux is evaluated once per face.  A face with a dry side takes the
// dry / wall branches, which are not antisymmetric (the wall branch keeps the
// dry side's xi; the one-side-dry branch uses the h-based pressure): each side
// is evaluated from its own cell, as the per-cell loop does.

// One side of a face, from the side records the face kernel forms once per
// cell: the pairs of xi and hstill, the clamped depth, the masked momenta and
// the velocity and sqrt(h) of own_f32.
struct FaceSideF32 {
  float xi, hst, h, hu, hv, u, v, s;
};

// Wet-wet Roe flux of side a (own pressure shift applied) through the face
// with unit normal n from a to b; returns dp = p_b - p_a (pressure_jump_f32).
// The algebra is roe_flux_wet_f32's, with b's velocity and sqrt(h) taken from
// its side record instead of being formed again.
__device__ __forceinline__ float roe_face_wet_f32(const FaceSideF32& A, const FaceSideF32& B, float dxi, float dhst,
                                                  float g, float nx, float ny, float F[3]) {
  const float rs = 1.0f / (A.s + B.s);
  const float uRoe = (A.s * A.u + B.s * B.u) * rs;
  const float vRoe = (A.s * A.v + B.s * B.v) * rs;
  const float unRoe = uRoe * nx + vRoe * ny;
  const float gh = g * ((A.h + B.h) * 0.5f);
  const float rc = rsqrtf(gh);
  const float cRoe = gh * rc;
  const float d1 = B.hu - A.hu, d2 = B.hv - A.hv;
  const float t = (unRoe * dxi - nx * d1 - ny * d2) * (0.5f * rc);
  const float w0 = (ny * d1 - nx * d2 - (uRoe * ny - vRoe * nx) * dxi) * smooth_abs_f32(unRoe);
  const float w1 = (0.5f * dxi + t) * smooth_abs_f32(unRoe - cRoe);
  const float w2 = (0.5f * dxi - t) * smooth_abs_f32(unRoe + cRoe);
  const float sum = w1 + w2, dif = cRoe * (w2 - w1);
  const float A1 = ny * w0 + uRoe * sum + nx * dif;
  const float A2 = -nx * w0 + vRoe * sum + ny * dif;
  const float dp = pressure_jump_f32(g, A.xi, B.xi, dxi, B.hst, dhst);
  F[0] = 0.5f * ((A.hu * nx + A.hv * ny) + (B.hu * nx + B.hv * ny) - sum);
  F[1] = 0.5f * (((A.hu * A.u + B.hu * B.u) + dp) * nx + (A.hu * A.v + B.hu * B.v) * ny - A1);
  F[2] = 0.5f * ((A.hv * A.u + B.hv * B.u) * nx + ((A.hv * A.v + B.hv * B.v) + dp) * ny - A2);
  return dp;
}

// Wet-wet HLL flux of side a (own pressure shift applied), hll_flux_wet_f32's
// algebra; returns dp = p_b - p_a.
__device__ __forceinline__ float hll_face_wet_f32(const FaceSideF32& A, const FaceSideF32& B, float dxi, float dhst,
                                                  float g, float nx, float ny, float F[3]) {
  const float rs = 1.0f / (A.s + B.s);
  const float uRoe = (A.s * A.u + B.s * B.u) * rs;
  const float vRoe = (A.s * A.v + B.s * B.v) * rs;
  const float unRoe = uRoe * nx + vRoe * ny;
  const float cRoe = sqrtf(g * ((A.h + B.h) * 0.5f));
  const float unL = A.u * nx + A.v * ny, unR = B.u * nx + B.v * ny;
  const float cL = sqrtf(g * A.h), cR = sqrtf(g * B.h);
  const float sL = fminf(unL - cL, unRoe - cRoe), sR = fmaxf(unR + cR, unRoe + cRoe);
  const float dp = pressure_jump_f32(g, A.xi, B.xi, dxi, B.hst, dhst);
  const float fL0 = A.hu * nx + A.hv * ny;
  const float fL1 = A.hu * A.u * nx + A.hu * A.v * ny;
  const float fL2 = A.hv * A.u * nx + A.hv * A.v * ny;
  const float fR0 = B.hu * nx + B.hv * ny;
  const float fR1 = B.hu * B.u * nx + B.hu * B.v * ny;
  const float fR2 = B.hv * B.u * nx + B.hv * B.v * ny;
  if (sL >= 0.0f) {
    F[0] = fL0; F[1] = fL1; F[2] = fL2;
  } else if (sR <= 0.0f) {
    F[0] = fR0; F[1] = fR1 + dp * nx; F[2] = fR2 + dp * ny;
  } else {
    const float r = 1.0f / (sR - sL), sLR = sL * sR;
    F[0] = (sR * fL0 - sL * fR0 + sLR * dxi) * r;
    F[1] = (sR * fL1 - sL * fR1 - sL * dp * nx + sLR * (B.hu - A.hu)) * r;
    F[2] = (sR * fL2 - sL * fR2 - sL * dp * ny + sLR * (B.hv - A.hv)) * r;
  }
  return dp;
}

}  // namespace hgd
