// Block-level reductions shared by the stage kernels.
#pragma once
#include <cmath>
#include <cstdint>

namespace hg {
namespace devred {

// Block-wide minimum of non-negative values, published with one atomicMin on
// the IEEE bit pattern (non-negative doubles order like unsigned integers), so
// the result does not depend on the order blocks finish in.
__device__ __forceinline__ void block_min_publish(double v, unsigned long long* out) {
  __shared__ double sm[32];
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sm[lane] : INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) atomicMin(out, (unsigned long long)__double_as_longlong(v));
  }
}

// FP32 variant: minimum of non-negative floats published on their bit pattern.
__device__ __forceinline__ void block_min_publish_f(float v, unsigned int* out) {
  __shared__ float smf[32];
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) smf[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? smf[lane] : INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) atomicMin(out, __float_as_uint(v));
  }
}

// Deterministic block sum (fixed thread -> element mapping, fixed tree).
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sm[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;   // valid in thread 0
}

// Block sum of floats as a double, deterministic, with one double formed per
// warp: each warp adds its lanes' values in a fixed float tree, carrying each
// addition's rounding error exactly (Knuth's TwoSum) in a second float, so the
// warp's sum has double-like accuracy without the FP64 pipe (a few FP64 adds a
// block instead of one per thread).
__device__ __forceinline__ double block_sum_f32(float v) {
  __shared__ double smw[32];
  float hi = v, lo = 0.0f;
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = __fadd_rn(hi, oh);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(oh, bp));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, ol), e);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smw[w] = (double)hi + (double)lo;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r += smw[k];
  return r;   // valid in thread 0
}

}  // namespace devred
}  // namespace hg
