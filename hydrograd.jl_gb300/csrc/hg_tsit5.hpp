// Tsitouras 5(4) Runge-Kutta pair (Ch. Tsitouras, "Runge-Kutta pairs of order
// 5(4) satisfying only the first column simplifying assumption", Computers &
// Mathematics with Applications 62 (2011) 770-775): the reference's default
// time integrator (Tsit5, swe_2D_forward_simulation.jl:37-39), restated from
// the published tableau.  The seventh stage is evaluated at the new state
// (first same as last), so an accepted step costs six RHS evaluations.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "hg_state.hpp"

namespace hg {

constexpr int kTsit5Stages = 7;
constexpr int kTsit5ErrorBlocks = 1024;   // grid of the combination / error kernels
// State vectors of the fixed-step Tsit5 adjoint (hg_adjoint.cpp): stage states
// Y_1..Y_5, stage RHS K_0..K_5, stage cotangents Ybar_0..Ybar_5, one Kbar.
constexpr int kTsit5Vectors = 18;

struct Tsit5Tableau {
  double c[kTsit5Stages];
  double a[kTsit5Stages][kTsit5Stages];   // a[i][j], j < i
  double b[kTsit5Stages];                 // 5th-order weights (= a[6][*], b[6] = 0)
  double btilde[kTsit5Stages];            // b - bhat (bhat: the embedded 4th-order weights)
};
const Tsit5Tableau& tsit5_tableau();

// Weighted vectors for one combination: sum_j w[j] K[j], j < nk.
struct Tsit5Terms {
  const double* K[kTsit5Stages];
  double w[kTsit5Stages];
  int nk;
};

void launch_tsit5_combine(int64_t len, const double* U, const Tsit5Terms& t, double dt, double* Y, cudaStream_t st);
// *norm2 = sum_i (dt sum_j w_j K_j[i] / (abstol + reltol max(|U_i|, |Unew_i|)))^2 (partials: kTsit5ErrorBlocks).
void launch_tsit5_error(int64_t len, const double* U, const double* Unew, const Tsit5Terms& t, double dt, double abstol,
                        double reltol, double* partials, unsigned int* ticket, double* norm2, cudaStream_t st);
// FP32-compensated contexts: the stage states are hi + lo records (StateF32),
// the stage RHS vectors [3n] floats, and the weights carry the step (w_j dt,
// rounded to float once).  The sums run in FP32 -- the RHS vectors hold
// FP32-accurate values -- and are added to the state with a compensated sum.
struct Tsit5TermsF {
  const float* K[kTsit5Stages];
  float w[kTsit5Stages];
  int nk;
};
// Y = U + sum_j w[j] K[j].
void launch_tsit5_combine_f32(int32_t n, StateF32 U, const Tsit5TermsF& t, StateF32 Y, cudaStream_t st);
// *norm2 = sum over the 3n values of (sum_j w_j K_j / (abstol + reltol max(|U|, |Unew|)))^2;
// with nk = 0 the values are U's own (the initial step's norm of the state).
void launch_tsit5_error_f32(int32_t n, StateF32 U, StateF32 Unew, const Tsit5TermsF& t, float abstol, float reltol,
                            double* partials, unsigned int* ticket, double* norm2, cudaStream_t st);
// Y = sum_j w[j] K[j] over float vectors of length len (the FP32-compensated
// Tsit5 adjoint's cotangent combinations).
void launch_tsit5_lin_f32(int64_t len, const Tsit5TermsF& t, float* Y, cudaStream_t st);
void launch_f32_to_f64(int32_t n, StateF32 X, double* Q, cudaStream_t st);
void launch_f64_to_f32(int32_t n, const double* Q, StateF32 X, cudaStream_t st);

}  // namespace hg
