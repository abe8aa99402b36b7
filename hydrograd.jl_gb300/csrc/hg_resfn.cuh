// Manning's n as a function of the state (process_ManningN_2D.jl:149-213),
// templated on the scalar: double and float for the resistance kernels, and
// the dual numbers of hg_dual.cuh for its derivatives in the adjoint (w.r.t.
// the cell's depth and velocity magnitude, and the function's parameters).
#pragma once
#include <cmath>

#include "hg_dual.cuh"
#include "hg_state.hpp"

namespace hgd {

template <class S>
struct RM;
template <>
struct RM<double> {
  static __device__ double exp(double x) { return ::exp(x); }
  static __device__ double tanh(double x) { return ::tanh(x); }
  static __device__ double log10(double x) { return ::log10(x); }
  static __device__ double log1p(double x) { return ::log1p(x); }
  static __device__ double pow(double x, double y) { return ::pow(x, y); }
  static __device__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ double abs(double x) { return ::fabs(x); }
  static __device__ double w(const hg::ResDev& r, int i) { return r.w[i]; }
  static __device__ double* hid(const hg::ResDev& r) { return r.hid; }
};
template <>
struct RM<float> {
  static __device__ float exp(float x) { return ::expf(x); }
  static __device__ float tanh(float x) { return ::tanhf(x); }
  static __device__ float log10(float x) { return ::log10f(x); }
  static __device__ float log1p(float x) { return ::log1pf(x); }
  static __device__ float pow(float x, float y) { return ::powf(x, y); }
  static __device__ float sqrt(float x) { return ::sqrtf(x); }
  static __device__ float abs(float x) { return ::fabsf(x); }
  static __device__ float w(const hg::ResDev& r, int i) { return r.wf[i]; }
  static __device__ float* hid(const hg::ResDev& r) { return r.hidF; }
};
// Dual numbers: each function's value by the scalar form above, its tangents
// by the chain rule.
template <class T, int N>
struct RM<Dn<T, N>> {
  using D = Dn<T, N>;
  static __device__ D scale(const D& a, T v, T k) {   // value v, tangents k a.d
    D r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = k * a.d[i];
    return r;
  }
  static __device__ D exp(const D& a) {
    const T e = RM<T>::exp(a.v);
    return scale(a, e, e);
  }
  static __device__ D log10(const D& a) { return scale(a, RM<T>::log10(a.v), T(0.43429448190325176) / a.v); }
  static __device__ D sqrt(const D& a) {
    const T s = RM<T>::sqrt(a.v);
    return scale(a, s, s > T(0) ? T(0.5) / s : T(0));
  }
  static __device__ D abs(const D& a) { return scale(a, RM<T>::abs(a.v), a.v < T(0) ? T(-1) : T(1)); }
  static __device__ D tanh(const D& a) {
    const T t = RM<T>::tanh(a.v);
    return scale(a, t, T(1) - t * t);
  }
  static __device__ D log1p(const D& a) { return scale(a, RM<T>::log1p(a.v), T(1) / (T(1) + a.v)); }
  // x^y: d = y x^(y-1) dx + x^y ln(x) dy (the second term only where x > 0)
  static __device__ D pow(const D& x, const D& y) {
    D r;
    r.v = RM<T>::pow(x.v, y.v);
    const T dx = y.v * RM<T>::pow(x.v, y.v - T(1));
    const T dy = x.v > T(0) ? r.v * ::log(x.v) : T(0);
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = dx * x.d[i] + dy * y.d[i];
    return r;
  }
};

// n(h, Umag, ks) with the parameters {n_lower, n_upper, k, h_mid} as p.
template <class S>
__device__ S manning_fn_p(int kind, const S (&p)[4], S h, S umag, S ks) {
  const S nl = p[0], nu = p[1], k = p[2];
  switch (kind) {
    case hg::kResPowerLaw: return nl + (nu - nl) * RM<S>::pow(h + S(2.220446049250313e-16), -k);
    case hg::kResSigmoid: return nl + (nu - nl) / (S(1) + RM<S>::exp(k * (h - p[3])));
    case hg::kResInverse: return nl + (nu - nl) / (S(1) + k * h);
    default: {   // h_Umag_ks: Cheng (2008) friction factor, Eq. 17
      const S Re = umag * h / S(1.0e-6);
      const S h_ks = h / ks;
      const S alpha = S(1) / (S(1) + RM<S>::pow(Re / S(850.0), S(9.0)));
      const S rb = Re / (h_ks * S(160.0));
      const S beta = S(1) / (S(1) + rb * rb);
      const S part1 = RM<S>::pow(Re / S(24.0), alpha);
      const S part2 = RM<S>::pow(S(1.8) * RM<S>::log10(Re / S(2.1)), S(2) * (S(1) - alpha) * beta);
      const S part3 = RM<S>::pow(S(2) * RM<S>::log10(S(11.8) * h_ks), S(2) * (S(1) - alpha) * (S(1) - beta));
      const S f = S(1) / (part1 * part2 * part3);
      return RM<S>::sqrt(f / S(8.0)) * RM<S>::pow(h, S(1.0 / 6.0)) / RM<S>::sqrt(S(9.81));
    }
  }
}

template <class S>
__device__ __forceinline__ S manning_fn(const hg::ResDev& r, S h, S umag, S ks) {
  const S p[4] = {S(r.p[0]), S(r.p[1]), S(r.p[2]), S(r.p[3])};
  return manning_fn_p<S>(r.kind, p, h, umag, ks);
}

// The derivatives of a cell's n (kinds power law .. h_Umag_ks) w.r.t. its
// clamped state -- depth h and momenta (qx, qy), through Umag = |q| / h --
// and w.r.t. the function's parameters: dn = dh dh' + dqx dqx' + dqy dqy' +
// sum_k dp[k] dp_k'.  A dry cell (h = h_small, q = 0) does not depend on its
// state.
template <class T>
struct ResJac {
  T n, dh, dqx, dqy, dp[4];
};
template <class T>
__device__ __forceinline__ ResJac<T> manning_jac(const hg::ResDev& r, T h, T qx, T qy, T ks, bool dry) {
  using D = Dn<T, 6>;   // tangents: h, Umag, p0..p3
  const T u = qx / h, v = qy / h;
  const T um = RM<T>::sqrt(u * u + v * v);
  const D p[4] = {D::seed(T(r.p[0]), 2), D::seed(T(r.p[1]), 3), D::seed(T(r.p[2]), 4), D::seed(T(r.p[3]), 5)};
  const D n = manning_fn_p<D>(r.kind, p, D::seed(h, 0), D::seed(um, 1), D(ks));
  ResJac<T> j;
  j.n = n.v;
#pragma unroll
  for (int k = 0; k < 4; ++k) j.dp[k] = n.d[2 + k];
  if (dry) {
    j.dh = j.dqx = j.dqy = T(0);
    return j;
  }
  // Umag = sqrt(u^2 + v^2), u = qx / h: dUmag/dqx = u / (Umag h), dUmag/dh = -Umag / h
  const T dnu = n.d[1];
  const T k = um > T(0) ? dnu / (um * h) : T(0);
  j.dh = n.d[0] - dnu * um / h;
  j.dqx = k * u;
  j.dqy = k * v;
  return j;
}

}  // namespace hgd
