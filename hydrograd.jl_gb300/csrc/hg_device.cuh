// Device-side arithmetic of the shallow-water RHS, templated on the scalar
// (double for the FP64 path, float for the FP32-compensated path).
//
// Follows src/fvm/discretization/Riemman_solvers/swe_2D_solvers.jl:4-164 (Roe
// flux with its dry/wet branches), src/utilities/smooth_functions.jl:4-52,
// src/fvm/boundary_conditions/bc_2D.jl:640-834 (ghost states) and
// src/fvm/discretization/semi_discretize_swe_2D.jl:449-559 (sources).
#pragma once
#include <cstdint>

namespace hgd {

// eps(Float64) from the smooth_* helpers.  The FP32 path keeps the FP64
// constant (as an FP32 literal): eps(Float32) would floor |u.n| near 3.4e-4.
template <class T> __device__ __forceinline__ T eps_c() { return T(2.220446049250313e-16); }

template <class T> __device__ __forceinline__ T smooth_abs(T x) { return sqrt(x * x + eps_c<T>()); }
template <class T> __device__ __forceinline__ T smooth_sqrt(T x) { return sqrt(x + eps_c<T>()); }
template <class T> __device__ __forceinline__ T smooth_pow2(T x) { T y = x + eps_c<T>(); return y * y; }

// xi of a dry cell: the largest xi with xi + hstill <= h_small in FP64, so the
// RHS sees the cell as dry.  h_small - hstill alone can round one ulp above
// h_small: a wet film 1e-19 m thick whose Manning friction (h + h_small)^(-7/3)
// breaks any explicit step.
__device__ __forceinline__ double prev_double(double x) {   // next representable double toward -inf (finite x)
  if (x == 0.0) return -4.9406564584124654e-324;
  const long long b = __double_as_longlong(x);
  return __longlong_as_double(x > 0.0 ? b - 1 : b + 1);
}
__device__ __forceinline__ double dry_xi(double hsm, double hst) {
  double x = __dsub_rn(hsm, hst);
  for (int i = 0; i < 4 && __dadd_rn(x, hst) > hsm; ++i) x = prev_double(x);
  return x;
}

// Boundary face encoding in the slot neighbour table.
constexpr int32_t kNoFace = INT32_MIN;
__device__ __forceinline__ bool is_boundary(int32_t nb) { return nb < 0; }
__device__ __forceinline__ int32_t boundary_index(int32_t nb) { return -1 - nb; }

enum : int32_t { kBcWall = 0, kBcSymm = 1, kBcInletQ = 2, kBcExitH = 3 };
// Riemann solvers of the faces (DevMesh::riemann, hg_set_riemann_solver).
enum : int32_t { kRiemannRoe = 0, kRiemannHll = 1 };

// One side of a face as the Roe solver sees it.
// `dry` is the reference's clamp decision h <= h_small (semi_discretize_swe_2D.jl:101-106).
// A clamped side has h == h_small and an unclamped side h > h_small, so the
// solver's `h <= hmin` tests are exactly `dry`; carrying the flag lets the FP32
// path take these decisions from its FP64-exact depth.
template <class T>
struct Side {
  T xi, hst, h, hu, hv, zb;
  bool dry;
};

// Roe flux through a face with unit normal (nx, ny) pointing from L to R.
// dxi = xiR - xiL is passed in so that the FP32 path can form it from its
// hi/lo state pairs without cancellation.
// bank: the wall test of a face with one dry side, (h_wet + zb_wet) <
// (zb_dry + hmin), taken by the caller (1 / 0), or -1: taken here from L and R.
// The FP32 path passes the FP64 decision (bank_wall_f64): with zb rounded to
// FP32 its own test would differ whenever a front's surface is within ~1e-7 m
// of the dry bank.
template <class T>
__device__ __forceinline__ void roe_flux(Side<T> L, Side<T> R, T dxi, T g, T nx, T ny, T hmin, T F[3],
                                         int bank = -1) {
  if (L.dry && R.dry) {                                   // both dry
    F[0] = T(0); F[1] = T(0); F[2] = T(0);
    return;
  } else if (R.dry && (bank >= 0 ? bank != 0 : (L.h + L.zb) < (R.zb + hmin))) {   // wall: R <- mirrored L (xiR kept)
    R.h = L.h; R.hu = -L.hu; R.hv = -L.hv;
  } else if (L.dry && (bank >= 0 ? bank != 0 : (R.h + R.zb) < (L.zb + hmin))) {   // wall: L <- mirrored R (xiL kept)
    L.h = R.h; L.hu = -R.hu; L.hv = -R.hv;
  } else if (L.dry) {                                     // left dry: physical flux of R, h-based pressure
    T p = T(0.5) * g * smooth_pow2(R.h);
    F[0] = R.hu * nx + R.hv * ny;
    F[1] = (R.hu * (R.hu / R.h) + p) * nx + R.hu * (R.hv / R.h) * ny;
    F[2] = (R.hv * (R.hu / R.h)) * nx + (R.hv * (R.hv / R.h) + p) * ny;
    return;
  } else if (R.dry) {                                     // right dry: physical flux of L
    T p = T(0.5) * g * smooth_pow2(L.h);
    F[0] = L.hu * nx + L.hv * ny;
    F[1] = (L.hu * (L.hu / L.h) + p) * nx + L.hu * (L.hv / L.h) * ny;
    F[2] = (L.hv * (L.hu / L.h)) * nx + (L.hv * (L.hv / L.h) + p) * ny;
    return;
  }
  const T uL = L.hu / L.h, vL = L.hv / L.h, uR = R.hu / R.h, vR = R.hv / R.h;
  const T sL = smooth_sqrt(L.h), sR = smooth_sqrt(R.h);
  const T hRoe = (L.h + R.h) / T(2);
  const T uRoe = (sL * uL + sR * uR) / (sL + sR);
  const T vRoe = (sL * vL + sR * vR) / (sL + sR);
  const T unRoe = uRoe * nx + vRoe * ny;
  const T cRoe = smooth_sqrt(g * hRoe);
  const T o2c = T(0.5) / cRoe;
  const T d1 = R.hu - L.hu, d2 = R.hv - L.hv;
  // w = |Lambda| (Lmat dQ), absA_dQ = Rmat w  (swe_2D_solvers.jl:103-118)
  T w0 = -(uRoe * ny - vRoe * nx) * dxi + ny * d1 + (-nx) * d2;
  T w1 = (unRoe * o2c + T(0.5)) * dxi + (-nx * o2c) * d1 + (-ny * o2c) * d2;
  T w2 = (-unRoe * o2c + T(0.5)) * dxi + (nx * o2c) * d1 + (ny * o2c) * d2;
  w0 *= smooth_abs(unRoe);
  w1 *= smooth_abs(unRoe - cRoe);
  w2 *= smooth_abs(unRoe + cRoe);
  const T A0 = w1 + w2;
  const T A1 = ny * w0 + (uRoe - cRoe * nx) * w1 + (uRoe + cRoe * nx) * w2;
  const T A2 = (-nx) * w0 + (vRoe - cRoe * ny) * w1 + (vRoe + cRoe * ny) * w2;
  // pre-balanced pressure 0.5 g (xi^2 + 2 xi hstill)  (swe_2D_solvers.jl:122-127)
  const T pL = T(0.5) * g * (smooth_pow2(L.xi) + T(2) * L.xi * L.hst);
  const T pR = T(0.5) * g * (smooth_pow2(R.xi) + T(2) * R.xi * R.hst);
  const T fL0 = L.hu * nx + L.hv * ny;
  const T fL1 = (L.hu * uL + pL) * nx + L.hu * vL * ny;
  const T fL2 = (L.hv * uL) * nx + (L.hv * vL + pL) * ny;
  const T fR0 = R.hu * nx + R.hv * ny;
  const T fR1 = (R.hu * uR + pR) * nx + R.hu * vR * ny;
  const T fR2 = (R.hv * uR) * nx + (R.hv * vR + pR) * ny;
  F[0] = (fL0 + fR0 - A0) / T(2);
  F[1] = (fL1 + fR1 - A1) / T(2);
  F[2] = (fL2 + fR2 - A2) / T(2);
}

// HLL flux -- new: the reference's RiemannSolver "HLL" raises an error
// (semi_discretize_swe_2D.jl:356-357).  Harten, Lax & van Leer (1983) with
// Einfeldt's (1988) wave speeds S_L = min(un_L - c_L, un_Roe - c_Roe),
// S_R = max(un_R + c_R, un_Roe + c_Roe), on roe_flux's variables (the
// pre-balanced pressure, the xi jump in the continuity row) and its dry, wall
// and one-side-dry branches; only the wet-wet flux differs:
//   F_L (S_L >= 0), F_R (S_R <= 0), else (S_R F_L - S_L F_R + S_L S_R dU) / (S_R - S_L).
template <class T>
__device__ __forceinline__ void hll_flux(Side<T> L, Side<T> R, T dxi, T g, T nx, T ny, T hmin, T F[3],
                                         int bank = -1) {
  if (L.dry && R.dry) {
    F[0] = T(0); F[1] = T(0); F[2] = T(0);
    return;
  } else if (R.dry && (bank >= 0 ? bank != 0 : (L.h + L.zb) < (R.zb + hmin))) {
    R.h = L.h; R.hu = -L.hu; R.hv = -L.hv;
  } else if (L.dry && (bank >= 0 ? bank != 0 : (R.h + R.zb) < (L.zb + hmin))) {
    L.h = R.h; L.hu = -R.hu; L.hv = -R.hv;
  } else if (L.dry) {
    T p = T(0.5) * g * smooth_pow2(R.h);
    F[0] = R.hu * nx + R.hv * ny;
    F[1] = (R.hu * (R.hu / R.h) + p) * nx + R.hu * (R.hv / R.h) * ny;
    F[2] = (R.hv * (R.hu / R.h)) * nx + (R.hv * (R.hv / R.h) + p) * ny;
    return;
  } else if (R.dry) {
    T p = T(0.5) * g * smooth_pow2(L.h);
    F[0] = L.hu * nx + L.hv * ny;
    F[1] = (L.hu * (L.hu / L.h) + p) * nx + L.hu * (L.hv / L.h) * ny;
    F[2] = (L.hv * (L.hu / L.h)) * nx + (L.hv * (L.hv / L.h) + p) * ny;
    return;
  }
  const T uL = L.hu / L.h, vL = L.hv / L.h, uR = R.hu / R.h, vR = R.hv / R.h;
  const T sqL = smooth_sqrt(L.h), sqR = smooth_sqrt(R.h);
  const T hRoe = (L.h + R.h) / T(2);
  const T uRoe = (sqL * uL + sqR * uR) / (sqL + sqR);
  const T vRoe = (sqL * vL + sqR * vR) / (sqL + sqR);
  const T unRoe = uRoe * nx + vRoe * ny;
  const T cRoe = smooth_sqrt(g * hRoe);
  const T unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
  const T cL = smooth_sqrt(g * L.h), cR = smooth_sqrt(g * R.h);
  const T sL1 = unL - cL, sL2 = unRoe - cRoe, sR1 = unR + cR, sR2 = unRoe + cRoe;
  const T sL = sL1 <= sL2 ? sL1 : sL2;
  const T sR = sR2 <= sR1 ? sR1 : sR2;
  const T pL = T(0.5) * g * (smooth_pow2(L.xi) + T(2) * L.xi * L.hst);
  const T pR = T(0.5) * g * (smooth_pow2(R.xi) + T(2) * R.xi * R.hst);
  const T fL0 = L.hu * nx + L.hv * ny;
  const T fL1 = (L.hu * uL + pL) * nx + L.hu * vL * ny;
  const T fL2 = (L.hv * uL) * nx + (L.hv * vL + pL) * ny;
  const T fR0 = R.hu * nx + R.hv * ny;
  const T fR1 = (R.hu * uR + pR) * nx + R.hu * vR * ny;
  const T fR2 = (R.hv * uR) * nx + (R.hv * vR + pR) * ny;
  if (!(sL < T(0))) {
    F[0] = fL0; F[1] = fL1; F[2] = fL2;
  } else if (sR <= T(0)) {
    F[0] = fR0; F[1] = fR1; F[2] = fR2;
  } else {
    const T den = sR - sL;
    F[0] = (sR * fL0 - sL * fR0 + sL * sR * dxi) / den;
    F[1] = (sR * fL1 - sL * fR1 + sL * sR * (R.hu - L.hu)) / den;
    F[2] = (sR * fL2 - sL * fR2 + sL * sR * (R.hv - L.hv)) / den;
  }
}

// The face flux of the context's Riemann solver (DevMesh::riemann); bank as in roe_flux.
template <class T>
__device__ __forceinline__ void riemann_flux(int solver, const Side<T>& L, const Side<T>& R, T dxi, T g, T nx, T ny,
                                             T hmin, T F[3], int bank = -1) {
  if (solver == kRiemannHll) hll_flux<T>(L, R, dxi, g, nx, ny, hmin, F, bank);
  else roe_flux<T>(L, R, dxi, g, nx, ny, hmin, F, bank);
}

// Ghost state of a boundary face (bc_2D.jl:640-834) from the clamped state of
// its internal cell L, the outward normal (nx, ny), and the boundary data.
// Returns R with R.xi = R.h - hstill (semi_discretize_swe_2D.jl:220), R.hst =
// hstill and R.zb = zb of the internal cell (update_ghost_cells_scalar).
template <class T>
__device__ __forceinline__ Side<T> ghost_state(const Side<T>& L, int32_t type, T nx, T ny, T hmin, T exitWse,
                                               T inletQ, T totalA, T lp23, T manning) {
  Side<T> R;
  R.hst = L.hst;
  R.zb = L.zb;
  R.h = L.h;
  R.dry = L.dry;
  if (type == kBcWall) {                       // (h, -qx, -qy)
    R.hu = -L.hu;
    R.hv = -L.hv;
  } else if (type == kBcSymm) {                // mirror the normal momentum
    T vdn = L.hu * nx + L.hv * ny;
    R.hu = L.hu - T(2) * vdn * nx;
    R.hv = L.hv - T(2) * vdn * ny;
  } else if (type == kBcExitH) {               // h = max(h_small, WSE - zb), q copied
    T hn = exitWse - L.zb;
    R.dry = !(hn > hmin);
    R.h = R.dry ? hmin : hn;
    R.hu = L.hu;
    R.hv = L.hv;
  } else {                                     // inlet-Q: q = -h v_n n_out wet, v_n = Q/total_A L^(2/3)/n
    T wet = L.dry ? T(0) : T(1);
    T vn = inletQ / totalA * lp23 / manning;
    R.hu = -L.h * vn * nx * wet;
    R.hv = -L.h * vn * ny * wet;
  }
  R.xi = R.h - R.hst;
  return R;
}

// Manning friction coefficient g n^2/k_n^2/(h+h_small)^(7/3) * smooth_sqrt(qx^2+qy^2)
// (semi_discretize_swe_2D.jl:544-547).
// FP64: (h + h_small)^(7/3) as x^2 cbrt(x) -- within a few 1e-16 of pow(x, 7/3)
// (the reference's ^(7/3)) for a fraction of pow's FP64 instructions, which GB300
// issues at 1/64 of its FP32 rate.
__device__ __forceinline__ double friction_coef(double g, double kn2, double hsm, double n, double h, double qx,
                                                double qy) {
  const double x = h + hsm;
  return g * (n * n) / kn2 / (x * x * cbrt(x)) * smooth_sqrt(qx * qx + qy * qy);
}
__device__ __forceinline__ float friction_coef(float g, float kn2, float hsm, float n, float h, float qx, float qy) {
  // (h + h_small)^(-7/3) = exp2(-7/3 log2(h + h_small))
  return g * (n * n) / kn2 * exp2f(-2.3333333333333335f * log2f(h + hsm)) * smooth_sqrt(qx * qx + qy * qy);
}

}  // namespace hgd
