// Hand-written reverse mode of the wet-wet Roe flux (both sides wet: the
// branch-free path of swe_2D_solvers.jl:79-164), templated on the scalar, for
// the VJP kernels of both paths.  The own cell's velocity, sqrt(h) and flux
// tensor adjoints are summed over its faces (roe_wet_vjp) and taken back to
// (xi, hu, hv) once (own_vjp).  The forward values are recomputed with the
// algebra regrouped (w1 + w2 = dxi exactly: w1 = dxi/2 + t, w2 = dxi/2 - t,
// t = (un dxi - nx d1 - ny d2) / (2c)); derivatives: smooth_abs(x)' =
// x / smooth_abs(x), smooth_sqrt(x)' = 1 / (2 smooth_sqrt(x)).
#pragma once

#include "hg_device.cuh"
#include "hg_f32.cuh"

namespace hgd {

// Per-precision primitives: sqrt(h + eps) and 1/h of a wet side, the Roe
// celerity c = sqrt(g hRoe + eps) and 1/(2c), smooth_abs.
template <class T> struct WetMath;

template <> struct WetMath<float> {
  // FP32: one reciprocal square root each (sqrt(h) = h r, 1/h = r^2); eps is
  // below FP32 resolution next to h > h_small, and smooth_abs(x) is |x| to
  // FP32 precision once |x| > 1e-4.
  static __device__ __forceinline__ void root_inv(float h, float& s, float& inv) {
    const float r = rsqrtf(h);
    s = h * r;
    inv = r * r;
  }
  static __device__ __forceinline__ void celerity(float gh, float& c, float& half_inv) {
    const float r = rsqrtf(gh);
    c = gh * r;
    half_inv = 0.5f * r;
  }
  static __device__ __forceinline__ float sabs(float x) { return smooth_abs_f32(x); }
};

template <> struct WetMath<double> {
  static __device__ __forceinline__ void root_inv(double h, double& s, double& inv) {
    s = smooth_sqrt(h);
    inv = 1.0 / h;
  }
  static __device__ __forceinline__ void celerity(double gh, double& c, double& half_inv) {
    c = smooth_sqrt(gh);
    half_inv = 0.5 / c;
  }
  static __device__ __forceinline__ double sabs(double x) { return smooth_abs(x); }
};

// The own cell's velocity and sqrt(h) (a wet side).
template <class T>
struct OwnV {
  T u, v, s;
};

template <class T>
__device__ __forceinline__ OwnV<T> own_v(const Side<T>& L) {
  OwnV<T> o;
  T inv;
  WetMath<T>::root_inv(L.h, o.s, inv);
  o.u = L.hu * inv;
  o.v = L.hv * inv;
  return o;
}

// Adjoints of the own cell's quantities, accumulated over its wet-wet faces by
// roe_wet_vjp and taken back to (xi, hu, hv) once by own_vjp.
template <class T>
struct OwnAdj {
  T u = T(0), v = T(0), s = T(0), fxx = T(0), fxy = T(0), fyx = T(0), fyy = T(0);
  T h = T(0), hu = T(0), hv = T(0), xi = T(0);
};

// Adds w . dF/d(own quantities) of one face to b; dxi = xiR - xiL.
template <class T>
__device__ __forceinline__ void roe_wet_vjp(const Side<T>& L, const OwnV<T>& o, const Side<T>& R, T dxi, T g, T nx,
                                            T ny, T w0, T w1, T w2, OwnAdj<T>& b) {
  using M = WetMath<T>;
  const T h = T(0.5);
  // forward
  T sR, rR;
  M::root_inv(R.h, sR, rR);
  const T uR = R.hu * rR, vR = R.hv * rR;
  const T rs = T(1) / (o.s + sR);
  const T numu = o.s * o.u + sR * uR, numv = o.s * o.v + sR * vR;
  const T uRoe = numu * rs, vRoe = numv * rs;
  const T un = uRoe * nx + vRoe * ny;
  T c, q;
  M::celerity(g * ((L.h + R.h) * h), c, q);
  const T d1 = R.hu - L.hu, d2 = R.hv - L.hv;
  const T Tt = un * dxi - nx * d1 - ny * d2;
  const T t = Tt * q;
  const T w0r = ny * d1 - nx * d2 - (uRoe * ny - vRoe * nx) * dxi;
  const T a0 = M::sabs(un), a1 = M::sabs(un - c), a2 = M::sabs(un + c);
  const T e1 = h * dxi + t, e2 = h * dxi - t;
  const T W1 = e1 * a1, W2 = e2 * a2;
  const T sum = W1 + W2;
  // reverse: F = (fL + fR - A) / 2
  const T bA0 = -h * w0, bA1 = -h * w1, bA2 = -h * w2;
  b.fxx += h * w1 * nx;
  b.fxy += h * w1 * ny;
  b.fyx += h * w2 * nx;
  b.fyy += h * w2 * ny;
  b.hu += h * w0 * nx;
  b.hv += h * w0 * ny;
  // A0 = sum, A1 = ny W0 + uRoe sum + nx dif, A2 = -nx W0 + vRoe sum + ny dif, dif = c (W2 - W1)
  const T bW0 = ny * bA1 - nx * bA2;
  const T bsum = bA0 + uRoe * bA1 + vRoe * bA2;
  const T bdif = nx * bA1 + ny * bA2;
  T buRoe = sum * bA1, bvRoe = sum * bA2;
  T bc = (W2 - W1) * bdif;
  const T bW1 = bsum - c * bdif, bW2 = bsum + c * bdif;
  // W0 = w0r a0, W1 = e1 a1, W2 = e2 a2
  const T bw0r = a0 * bW0;
  const T ba0 = w0r * bW0, ba1 = e1 * bW1, ba2 = e2 * bW2;
  const T bt = a1 * bW1 - a2 * bW2;
  T bdxi = h * (a1 * bW1 + a2 * bW2);
  const T r0 = un / a0, r1 = (un - c) / a1, r2 = (un + c) / a2;
  T bun = ba0 * r0 + ba1 * r1 + ba2 * r2;
  bc += ba2 * r2 - ba1 * r1;
  // w0r = ny d1 - nx d2 - (uRoe ny - vRoe nx) dxi
  T bd1 = ny * bw0r, bd2 = -nx * bw0r;
  buRoe -= ny * dxi * bw0r;
  bvRoe += nx * dxi * bw0r;
  bdxi -= (uRoe * ny - vRoe * nx) * bw0r;
  // t = Tt q, q = 1 / (2 c), Tt = un dxi - nx d1 - ny d2
  const T bT = q * bt;
  bc -= Tt * bt * q / c;
  bun += dxi * bT;
  bdxi += un * bT;
  bd1 -= nx * bT;
  bd2 -= ny * bT;
  b.hu -= bd1;
  b.hv -= bd2;
  // c = smooth_sqrt(g (hL + hR) / 2)
  b.h += h * g * q * bc;
  // un = uRoe nx + vRoe ny; uRoe = numu rs, rs = 1 / (s + sR)
  buRoe += nx * bun;
  bvRoe += ny * bun;
  const T bnumu = rs * buRoe, bnumv = rs * bvRoe;
  const T brs = numu * buRoe + numv * bvRoe;
  b.s += o.u * bnumu + o.v * bnumv - rs * rs * brs;
  b.u += o.s * bnumu;
  b.v += o.s * bnumv;
  b.xi -= bdxi;
}

// Takes the accumulated adjoints back to the own state: d/d(xi, hu, hv).  The
// flux tensor is the reference's, with the own pressure in it: fxx = hu u + p,
// fxy = hu v, fyx = hv u, fyy = hv v + p, p = g/2 (smooth_pow2(xi) +
// 2 xi hstill).  (The FP32 forward pass's p_L n shift sums to zero over the
// cell's faces.)
template <class T>
__device__ __forceinline__ void own_vjp(const Side<T>& L, const OwnV<T>& o, T g, OwnAdj<T> b, T& gxi, T& ghu, T& ghv) {
  b.hu += o.u * b.fxx + o.v * b.fxy;
  b.hv += o.u * b.fyx + o.v * b.fyy;
  b.u += L.hu * b.fxx + L.hv * b.fyx;
  b.v += L.hu * b.fxy + L.hv * b.fyy;
  const T bp = b.fxx + b.fyy;
  b.xi += bp * g * ((L.xi + eps_c<T>()) + L.hst);
  // s = smooth_sqrt(h); u = hu / h, v = hv / h; h = xi + hstill
  const T rh = T(1) / L.h;
  b.h += b.s * T(0.5) / o.s;
  b.hu += b.u * rh;
  b.hv += b.v * rh;
  b.h -= (b.u * o.u + b.v * o.v) * rh;
  gxi = b.xi + b.h;
  ghu = b.hu;
  ghv = b.hv;
}

}  // namespace hgd
