// Device kernels of the Tsit5 integrator (hg_tsit5.cpp): stage combinations,
// the error norm, and conversions between the FP32-compensated state records
// and plain FP64 state vectors.  All vectors are [3n] doubles in the device
// cell order.
#include <cmath>

#include "hg_reduce.cuh"
#include "hg_state.hpp"
#include "hg_tsit5.hpp"

namespace hg {

using namespace devred;

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

void launch_f32_to_f64(int32_t n, StateF32 X, double* Q, cudaStream_t st) {
  k_f32_to_f64<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(n, X, Q);
}

void launch_f64_to_f32(int32_t n, const double* Q, StateF32 X, cudaStream_t st) {
  k_f64_to_f32<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(n, Q, X);
}

}  // namespace hg
