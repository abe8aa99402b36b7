// Device kernels of the Tsit5 integrator (hg_tsit5.cpp): stage combinations,
// the error norm, and conversions between the FP32-compensated state records
// and plain FP64 state vectors.  All vectors are [3n] doubles in the device
// cell order.
#include <cmath>

#include "hg_f32.cuh"
#include "hg_reduce.cuh"
#include "hg_state.hpp"
#include "hg_tsit5.hpp"

namespace hg {

using namespace devred;
using hgd::df_add;

namespace {

constexpr int kBlock = 256;

// Y = U + dt sum_j w[j] K[j] over the nk vectors in K (U null: Y = dt sum).
__global__ void __launch_bounds__(kBlock) k_tsit5_combine(int64_t len, const double* __restrict__ U, Tsit5Terms t,
                                                          double dt, double* __restrict__ Y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kTsit5Stages; ++j)
      if (j < t.nk) s += t.w[j] * t.K[j][i];
    Y[i] = U ? U[i] + dt * s : dt * s;
  }
}

// Per block: sum of (E_i / (abstol + reltol max(|U_i|, |Unew_i|)))^2 with
// E = dt sum_j btilde_j K_j; the last block to finish adds the partials in
// block order (deterministic) into *norm2.
__global__ void __launch_bounds__(kBlock) k_tsit5_error(int64_t len, const double* __restrict__ U,
                                                        const double* __restrict__ Unew, Tsit5Terms t, double dt,
                                                        double abstol, double reltol, double* partials,
                                                        unsigned int* ticket, double* norm2) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    double e = 0.0;
#pragma unroll
    for (int j = 0; j < kTsit5Stages; ++j)
      if (j < t.nk) e += t.w[j] * t.K[j][i];
    e *= dt;
    const double sc = abstol + reltol * fmax(fabs(U[i]), fabs(Unew[i]));
    const double r = e / sc;
    acc += r * r;
  }
  const double b = block_sum(acc);
  __shared__ int isLast;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    isLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!isLast) return;
  __threadfence();
  double s = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) s += __ldcg(&partials[k]);
  const double tot = block_sum(s);
  if (threadIdx.x == 0) {
    *norm2 = tot;
    *ticket = 0u;
  }
}

// FP32-compensated stage state: Y = U + sum_j w_j K_j per cell, the sums in
// FP32 in stage order, added to the hi + lo pairs exactly (df_add).
__global__ void __launch_bounds__(kBlock) k_tsit5_combine_f32(int32_t n, StateF32 U, Tsit5TermsF t, StateF32 Y) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int j = 0; j < kTsit5Stages; ++j)
      if (j < t.nk) {
        const float w = t.w[j];
        const float* __restrict__ K = t.K[j];
        s0 = fmaf(w, __ldg(&K[c]), s0);
        s1 = fmaf(w, __ldg(&K[n + c]), s1);
        s2 = fmaf(w, __ldg(&K[2 * n + c]), s2);
      }
    const float4 u = U.x[c];
    const float2 q = U.q[c];
    float xh, xl, uh, ul, vh, vl;
    df_add(u.x, u.y, s0, xh, xl);
    df_add(u.z, q.x, s1, uh, ul);
    df_add(u.w, q.y, s2, vh, vl);
    Y.x[c] = make_float4(xh, xl, uh, vh);
    Y.q[c] = make_float2(ul, vl);
  }
}

// The weighted RMS terms of an FP32-compensated run, in FP32 per value and
// per thread, the block sums carried exactly to double (block_sum_f32); the
// last block adds the partials in block order.
__global__ void __launch_bounds__(kBlock) k_tsit5_error_f32(int32_t n, StateF32 U, StateF32 Unew, Tsit5TermsF t,
                                                            float abstol, float reltol, double* partials,
                                                            unsigned int* ticket, double* norm2) {
  float acc = 0.0f;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const float4 u = U.x[c], un = Unew.x[c];
    const float2 q = U.q[c];
    float e[3] = {0.0f, 0.0f, 0.0f};
    if (t.nk == 0) {   // the state itself
      e[0] = u.x + u.y;
      e[1] = u.z + q.x;
      e[2] = u.w + q.y;
    }
#pragma unroll
    for (int j = 0; j < kTsit5Stages; ++j)
      if (j < t.nk) {
        const float w = t.w[j];
        const float* __restrict__ K = t.K[j];
        e[0] = fmaf(w, __ldg(&K[c]), e[0]);
        e[1] = fmaf(w, __ldg(&K[n + c]), e[1]);
        e[2] = fmaf(w, __ldg(&K[2 * n + c]), e[2]);
      }
    const float a[3] = {u.x, u.z, u.w}, b[3] = {un.x, un.z, un.w};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float r = e[k] / (abstol + reltol * fmaxf(fabsf(a[k]), fabsf(b[k])));
      acc = fmaf(r, r, acc);
    }
  }
  const double b = block_sum_f32(acc);
  __shared__ int isLast;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    isLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!isLast) return;
  __threadfence();
  double s = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) s += __ldcg(&partials[k]);
  const double tot = block_sum(s);
  if (threadIdx.x == 0) {
    *norm2 = tot;
    *ticket = 0u;
  }
}

__global__ void __launch_bounds__(kBlock) k_tsit5_lin_f32(int64_t len, Tsit5TermsF t, float* __restrict__ Y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < kTsit5Stages; ++j)
      if (j < t.nk) s = fmaf(t.w[j], __ldg(&t.K[j][i]), s);
    Y[i] = s;
  }
}

__global__ void k_f32_to_f64(int32_t n, StateF32 X, double* __restrict__ Q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = X.x[i];
  const float2 q = X.q[i];
  Q[i] = (double)x.x + (double)x.y;
  Q[n + i] = (double)x.z + (double)q.x;
  Q[2 * n + i] = (double)x.w + (double)q.y;
}

__global__ void k_f64_to_f32(int32_t n, const double* __restrict__ Q, StateF32 X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float h[3], l[3];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const double v = Q[(size_t)b * n + i];
    h[b] = (float)v;
    l[b] = (float)(v - (double)h[b]);
  }
  X.x[i] = make_float4(h[0], l[0], h[1], h[2]);
  X.q[i] = make_float2(l[1], l[2]);
}

int grid_for(int64_t len) {
  const int64_t b = (len + kBlock - 1) / kBlock;
  return (int)(b < kTsit5ErrorBlocks ? b : kTsit5ErrorBlocks);
}

}  // namespace

void launch_tsit5_combine(int64_t len, const double* U, const Tsit5Terms& t, double dt, double* Y, cudaStream_t st) {
  k_tsit5_combine<<<grid_for(len), kBlock, 0, st>>>(len, U, t, dt, Y);
}

void launch_tsit5_error(int64_t len, const double* U, const double* Unew, const Tsit5Terms& t, double dt, double abstol,
                        double reltol, double* partials, unsigned int* ticket, double* norm2, cudaStream_t st) {
  k_tsit5_error<<<grid_for(len), kBlock, 0, st>>>(len, U, Unew, t, dt, abstol, reltol, partials, ticket, norm2);
}

void launch_tsit5_combine_f32(int32_t n, StateF32 U, const Tsit5TermsF& t, StateF32 Y, cudaStream_t st) {
  k_tsit5_combine_f32<<<grid_for(n), kBlock, 0, st>>>(n, U, t, Y);
}

void launch_tsit5_error_f32(int32_t n, StateF32 U, StateF32 Unew, const Tsit5TermsF& t, float abstol, float reltol,
                            double* partials, unsigned int* ticket, double* norm2, cudaStream_t st) {
  k_tsit5_error_f32<<<grid_for(n), kBlock, 0, st>>>(n, U, Unew, t, abstol, reltol, partials, ticket, norm2);
}

void launch_tsit5_lin_f32(int64_t len, const Tsit5TermsF& t, float* Y, cudaStream_t st) {
  k_tsit5_lin_f32<<<grid_for(len), kBlock, 0, st>>>(len, t, Y);
}

void launch_f32_to_f64(int32_t n, StateF32 X, double* Q, cudaStream_t st) {
  k_f32_to_f64<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(n, X, Q);
}

void launch_f64_to_f32(int32_t n, const double* Q, StateF32 X, cudaStream_t st) {
  k_f64_to_f32<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(n, Q, X);
}

}  // namespace hg
