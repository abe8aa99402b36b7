// Forward-mode dual numbers for the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Dual<N> carries a value and N tangent components,
// propagated by the chain rule the way ForwardDiff.jl's Dual does (ForwardDiff
// 0.10.38 is the version Hydrograd.jl's Project.toml pins).  Branches compare
// values only, as ForwardDiff's comparison operators do.
#pragma once
#include <cmath>

namespace hgo {

inline double value(double x) { return x; }

template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
  Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0.0; }   // NOLINT: implicit on purpose
};

template <int N> inline double value(const Dual<N>& x) { return x.v; }

template <int N> inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v;
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  double inv = 1.0 / b.v;
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v / b;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }

template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r; r.v = std::sqrt(a.v);
  double k = 0.5 / r.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k;
  return r;
}
template <int N> inline Dual<N> pow(const Dual<N>& a, double p) {
  Dual<N> r; r.v = std::pow(a.v, p);
  double k = p * std::pow(a.v, p - 1.0);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k;
  return r;
}

}  // namespace hgo
