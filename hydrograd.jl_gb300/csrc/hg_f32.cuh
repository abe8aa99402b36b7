// FP32-compensated path: packed cell records, the FP64-exact dry decision and
// double-float (hi + lo) arithmetic, shared by the forward and adjoint kernels.
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

}  // namespace hgd
