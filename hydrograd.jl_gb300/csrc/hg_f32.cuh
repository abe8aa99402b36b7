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

// Adjoints of the own cell's quantities, accumulated over its wet-wet faces by
// roe_wet_vjp_f32 and taken back to (xi, hu, hv) once by own_vjp_f32.
struct OwnAdjF32 {
  float u = 0.0f, v = 0.0f, s = 0.0f, fxx = 0.0f, fxy = 0.0f, fyx = 0.0f, fyy = 0.0f;
  float h = 0.0f, hu = 0.0f, hv = 0.0f, xi = 0.0f;
};

// Reverse mode of roe_flux_wet_f32 in the own (left) side: adds
// w . dF/d(own quantities) to b, with dxi = (xiR - xiL) + (lo parts).  The
// forward values are recomputed here; the reverse sweep follows them in
// reverse order (smooth_abs(x)' = x / smooth_abs(x), smooth_sqrt(x)' =
// 1 / (2 smooth_sqrt(x))).
__device__ __forceinline__ void roe_wet_vjp_f32(const Side<float>& L, const OwnF32& o, const Side<float>& R,
                                                float dxi, float g, float nx, float ny, float w0, float w1, float w2,
                                                OwnAdjF32& b) {
  // forward
  const float rq = rsqrtf(R.h);
  const float rR = rq * rq;
  const float uR = R.hu * rR, vR = R.hv * rR;
  const float sR = R.h * rq;
  const float rs = 1.0f / (o.s + sR);
  const float numu = o.s * o.u + sR * uR, numv = o.s * o.v + sR * vR;
  const float uRoe = numu * rs, vRoe = numv * rs;
  const float un = uRoe * nx + vRoe * ny;
  const float gh = g * ((L.h + R.h) * 0.5f);
  const float rc = rsqrtf(gh);
  const float c = gh * rc;
  const float q = 0.5f * rc;
  const float d1 = R.hu - L.hu, d2 = R.hv - L.hv;
  const float T = un * dxi - nx * d1 - ny * d2;
  const float t = T * q;
  const float w0r = ny * d1 - nx * d2 - (uRoe * ny - vRoe * nx) * dxi;
  const float a0 = smooth_abs_f32(un), a1 = smooth_abs_f32(un - c), a2 = smooth_abs_f32(un + c);
  const float e1 = 0.5f * dxi + t, e2 = 0.5f * dxi - t;
  const float W1 = e1 * a1, W2 = e2 * a2;
  const float sum = W1 + W2;
  // reverse: F = (fL + fR - A) / 2
  const float bA0 = -0.5f * w0, bA1 = -0.5f * w1, bA2 = -0.5f * w2;
  b.fxx += 0.5f * w1 * nx;
  b.fxy += 0.5f * w1 * ny;
  b.fyx += 0.5f * w2 * nx;
  b.fyy += 0.5f * w2 * ny;
  b.hu += 0.5f * w0 * nx;
  b.hv += 0.5f * w0 * ny;
  // A0 = sum, A1 = ny W0 + uRoe sum + nx dif, A2 = -nx W0 + vRoe sum + ny dif, dif = c (W2 - W1)
  const float bW0 = ny * bA1 - nx * bA2;
  const float bsum = bA0 + uRoe * bA1 + vRoe * bA2;
  const float bdif = nx * bA1 + ny * bA2;
  float buRoe = sum * bA1, bvRoe = sum * bA2;
  float bc = (W2 - W1) * bdif;
  const float bW1 = bsum - c * bdif, bW2 = bsum + c * bdif;
  // W0 = w0r a0, W1 = e1 a1, W2 = e2 a2
  const float bw0r = a0 * bW0;
  const float ba0 = w0r * bW0, ba1 = e1 * bW1, ba2 = e2 * bW2;
  const float bt = a1 * bW1 - a2 * bW2;
  float bdxi = 0.5f * (a1 * bW1 + a2 * bW2);
  const float r0 = un / a0, r1 = (un - c) / a1, r2 = (un + c) / a2;
  float bun = ba0 * r0 + ba1 * r1 + ba2 * r2;
  bc += ba2 * r2 - ba1 * r1;
  // w0r = ny d1 - nx d2 - (uRoe ny - vRoe nx) dxi
  float bd1 = ny * bw0r, bd2 = -nx * bw0r;
  buRoe -= ny * dxi * bw0r;
  bvRoe += nx * dxi * bw0r;
  bdxi -= (uRoe * ny - vRoe * nx) * bw0r;
  // t = T q, q = 1 / (2 c), T = un dxi - nx d1 - ny d2
  const float bT = q * bt;
  bc -= T * bt * q / c;
  bun += dxi * bT;
  bdxi += un * bT;
  bd1 -= nx * bT;
  bd2 -= ny * bT;
  b.hu -= bd1;
  b.hv -= bd2;
  // c = smooth_sqrt(g (hL + hR) / 2)
  b.h += 0.5f * g * q * bc;
  // un = uRoe nx + vRoe ny; uRoe = numu rs, rs = 1 / (s + sR)
  buRoe += nx * bun;
  bvRoe += ny * bun;
  const float bnumu = rs * buRoe, bnumv = rs * bvRoe;
  const float brs = numu * buRoe + numv * bvRoe;
  b.s += o.u * bnumu + o.v * bnumv - rs * rs * brs;
  b.u += o.s * bnumu;
  b.v += o.s * bnumv;
  b.xi -= bdxi;
}

// Takes the accumulated adjoints of the own quantities (own_f32) back to the
// own state: returns d/d(xi, hu, hv).
__device__ __forceinline__ void own_vjp_f32(const Side<float>& L, const OwnF32& o, float g, OwnAdjF32 b, float& gxi,
                                            float& ghu, float& ghv) {
  // Derivative of the reference flux, with the own pressure in the tensor:
  // fxx = hu u + p, fxy = hu v, fyx = hv u, fyy = hv v + p.  (The forward
  // pass's p_L n shift sums to zero over the cell's faces.)
  b.hu += o.u * b.fxx + o.v * b.fxy;
  b.hv += o.u * b.fyx + o.v * b.fyy;
  b.u += L.hu * b.fxx + L.hv * b.fyx;
  b.v += L.hu * b.fxy + L.hv * b.fyy;
  const float bp = b.fxx + b.fyy;
  // p = g/2 (smooth_pow2(xi) + 2 xi hstill)
  b.xi += bp * g * ((L.xi + eps_c<float>()) + L.hst);
  // s = smooth_sqrt(h); u = hu / h, v = hv / h; h = xi + hstill
  const float rh = 1.0f / L.h;
  b.h += b.s * 0.5f / o.s;
  b.hu += b.u * rh;
  b.hv += b.v * rh;
  b.h -= (b.u * o.u + b.v * o.v) * rh;
  gxi = b.xi + b.h;
  ghu = b.hu;
  ghv = b.hv;
}

}  // namespace hgd
