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

// Packed FP32x2 arithmetic (Blackwell's paired FP32 instructions: one issue
// slot for two lanes of the same operation, each rounded as its scalar form).
// The stage kernels are bound by instruction issue, and most of their FP32
// work comes in pairs -- the (qx, qy) rows of the update, (u, v), the momentum
// rows of a flux -- so the pairs are written with these.
__device__ __forceinline__ float2 p2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 p2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// two_sum / fast_two_sum / df_add / df_add2 on two lanes at once.
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  const float2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  e = sub2(b, sub2(s, a));
}
__device__ __forceinline__ void df_add_2(float2 ah, float2 al, float2 d, float2& rh, float2& rl) {
  float2 s, e;
  two_sum2(ah, d, s, e);
  e = add2(e, al);
  fast_two_sum2(s, e, rh, rl);
}
__device__ __forceinline__ void df_add2_2(float2 ah, float2 al, float2 bh, float2 bl, float2& rh, float2& rl) {
  float2 s, e;
  two_sum2(ah, bh, s, e);
  e = add2(e, add2(al, bl));
  fast_two_sum2(s, e, rh, rl);
}

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

// The Riemann solvers' wall test of a face whose sides differ in wetness,
// (h_w + zb_w) < (zb_d + h_small) with w the wet cell and d the dry one
// (swe_2D_solvers.jl:23-53), taken in FP64 as the FP64 path takes it: h_w from
// the wet cell's xi pair and the FP64 hstill, both beds from the FP64 zb.  The
// cell records hold zb in FP32 (rounded by up to 2.4e-7 m at 2-5 m of bed),
// and an FP32 test would differ from the FP64 one whenever a front's surface is
// within that distance of the dry bank -- for about one step of most front
// crossings -- so that the two precisions flood a dry cell on different steps
// and their states part at the fronts.  Faces with one dry side are few (the
// fronts), so the FP64 loads and arithmetic cost nothing measurable.
__device__ __forceinline__ int bank_wall_f64(const hg::DevMesh& m, float xh, float xl, int w, int d) {
  const double hw = ((double)xh + (double)xl) + __ldg(&m.hst[w]);
  return (hw + __ldg(&m.zb[w])) < (__ldg(&m.zb[d]) + m.hsm) ? 1 : 0;
}
// The same test for an exit-H face of cell c whose ghost is wet and c dry:
// the ghost's depth WSE - zb (bc_2D.jl exit-H ghost) against its own bed.
__device__ __forceinline__ int bank_exit_f64(const hg::DevMesh& m, int grp, int c) {
  const double zb = __ldg(&m.zb[c]);
  return ((m.exitWse[grp] - zb) + zb) < (zb + m.hsm) ? 1 : 0;
}

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
  const float2 qL = p2(L.hu, L.hv), qR = p2(R.hu, R.hv);
  const float2 uvR = mul2(qR, p2(rR));   // (uR, vR)
  const float sR = R.h * rq;
  const float rs = 1.0f / (o.s + sR);
  const float2 uvRoe = mul2(fma2(p2(o.s), p2(o.u, o.v), mul2(p2(sR), uvR)), p2(rs));
  const float unRoe = uvRoe.x * nx + uvRoe.y * ny;
  const float gh = g * ((L.h + R.h) * 0.5f);
  const float rc = rsqrtf(gh);
  const float cRoe = gh * rc;   // sqrt(g hRoe)
  const float2 d = sub2(qR, qL);   // (d1, d2)
  const float t = (unRoe * dxi - nx * d.x - ny * d.y) * (0.5f * rc);
  const float w0 = (ny * d.x - nx * d.y - (uvRoe.x * ny - uvRoe.y * nx) * dxi) * smooth_abs_f32(unRoe);
  const float w1 = (0.5f * dxi + t) * smooth_abs_f32(unRoe - cRoe);
  const float w2 = (0.5f * dxi - t) * smooth_abs_f32(unRoe + cRoe);
  const float sum = w1 + w2, dif = cRoe * (w2 - w1);
  // (A1, A2) = (ny, -nx) w0 + (uRoe, vRoe) sum + (nx, ny) dif
  const float2 A12 = fma2(p2(ny, -nx), p2(w0), fma2(uvRoe, p2(sum), mul2(p2(nx, ny), p2(dif))));
  const float dp = pressure_jump_f32(g, L.xi, R.xi, dxi, R.hst, dhst);   // p_R - p_L
  // momentum rows: own tensor . n, the other side's tensor . n, plus dp n
  const float2 fLn = fma2(p2(o.fxx, o.fyx), p2(nx), mul2(p2(o.fxy, o.fyy), p2(ny)));
  const float2 fRn = fma2(mul2(qR, p2(uvR.x)), p2(nx), fma2(mul2(qR, p2(uvR.y)), p2(ny), mul2(p2(dp), p2(nx, ny))));
  F[0] = 0.5f * ((L.hu * nx + L.hv * ny) + (R.hu * nx + R.hv * ny) - sum);
  const float2 F12 = mul2(p2(0.5f), sub2(add2(fLn, fRn), A12));
  F[1] = F12.x;
  F[2] = F12.y;
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
  const float2 uvA = p2(A.u, A.v), uvB = p2(B.u, B.v);
  const float2 qA = p2(A.hu, A.hv), qB = p2(B.hu, B.hv);
  const float2 uvRoe = mul2(fma2(p2(A.s), uvA, mul2(p2(B.s), uvB)), p2(rs));
  const float unRoe = uvRoe.x * nx + uvRoe.y * ny;
  const float gh = g * ((A.h + B.h) * 0.5f);
  const float rc = rsqrtf(gh);
  const float cRoe = gh * rc;
  const float2 d = sub2(qB, qA);
  const float t = (unRoe * dxi - nx * d.x - ny * d.y) * (0.5f * rc);
  const float w0 = (ny * d.x - nx * d.y - (uvRoe.x * ny - uvRoe.y * nx) * dxi) * smooth_abs_f32(unRoe);
  const float w1 = (0.5f * dxi + t) * smooth_abs_f32(unRoe - cRoe);
  const float w2 = (0.5f * dxi - t) * smooth_abs_f32(unRoe + cRoe);
  const float sum = w1 + w2, dif = cRoe * (w2 - w1);
  const float2 A12 = fma2(p2(ny, -nx), p2(w0), fma2(uvRoe, p2(sum), mul2(p2(nx, ny), p2(dif))));
  const float dp = pressure_jump_f32(g, A.xi, B.xi, dxi, B.hst, dhst);
  // (hu u, hv u) and (hu v, hv v) of both sides, dotted with n, plus dp n
  const float2 fu = fma2(qA, p2(uvA.x), mul2(qB, p2(uvB.x)));
  const float2 fv = fma2(qA, p2(uvA.y), mul2(qB, p2(uvB.y)));
  const float2 fn = fma2(fu, p2(nx), fma2(fv, p2(ny), mul2(p2(dp), p2(nx, ny))));
  F[0] = 0.5f * ((A.hu * nx + A.hv * ny) + (B.hu * nx + B.hv * ny) - sum);
  const float2 F12 = mul2(p2(0.5f), sub2(fn, A12));
  F[1] = F12.x;
  F[2] = F12.y;
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
