// Forward-mode dual numbers for the adjoint kernels.
//
// Dn<T, N> carries a value and N tangent components.  The adjoint kernels
// evaluate the same templated Roe flux / ghost-state code as the forward pass
// (hg_device.cuh) on Dn operands seeded on one cell's state (and, on boundary
// faces, on the parameters that enter the ghost state) to get exact local
// Jacobians, which they contract with the adjoint weights.  Comparisons use
// the value only, so every branch is the one the forward pass took.
#pragma once

namespace hgd {

using ::sqrt;   // keep the scalar overloads visible next to the dual one below

template <class T, int N>
struct Dn {
  T v;
  T d[N];
  __device__ __forceinline__ Dn() {}
  __device__ __forceinline__ Dn(double x) : v(T(x)) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = T(0);
  }
  __device__ __forceinline__ Dn(float x) : v(T(x)) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = T(0);
  }
  __device__ __forceinline__ Dn(int x) : v(T(x)) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = T(0);
  }
  // value x with tangent e_k (k < 0: no tangent)
  __device__ __forceinline__ static Dn seed(T x, int k) {
    Dn r(x);
    if (k >= 0) r.d[k] = T(1);
    return r;
  }
  __device__ __forceinline__ Dn& operator*=(const Dn& b);
};

#define HGD_DN template <class T, int N> __device__ __forceinline__

HGD_DN Dn<T, N> operator-(const Dn<T, N>& a) {
  Dn<T, N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
HGD_DN Dn<T, N> operator+(const Dn<T, N>& a, const Dn<T, N>& b) {
  Dn<T, N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
HGD_DN Dn<T, N> operator-(const Dn<T, N>& a, const Dn<T, N>& b) {
  Dn<T, N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
HGD_DN Dn<T, N> operator*(const Dn<T, N>& a, const Dn<T, N>& b) {
  Dn<T, N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
HGD_DN Dn<T, N> operator/(const Dn<T, N>& a, const Dn<T, N>& b) {
  Dn<T, N> r; r.v = a.v / b.v;
  const T inv = T(1) / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
template <class T, int N>
__device__ __forceinline__ Dn<T, N>& Dn<T, N>::operator*=(const Dn<T, N>& b) {
  *this = *this * b;
  return *this;
}
HGD_DN Dn<T, N> sqrt(const Dn<T, N>& a) {
  Dn<T, N> r; r.v = ::sqrt(a.v);
  const T k = T(0.5) / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k;
  return r;
}
HGD_DN bool operator<(const Dn<T, N>& a, const Dn<T, N>& b) { return a.v < b.v; }
HGD_DN bool operator<=(const Dn<T, N>& a, const Dn<T, N>& b) { return a.v <= b.v; }
HGD_DN bool operator>(const Dn<T, N>& a, const Dn<T, N>& b) { return a.v > b.v; }

#undef HGD_DN

}  // namespace hgd
