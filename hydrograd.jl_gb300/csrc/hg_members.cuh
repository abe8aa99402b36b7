// Per-member time steps of an ensemble (DevScalars::nMembers > 0): the member
// of a cell, and CFL candidates published into each member's own minimum.
// Members own contiguous device cell ranges (each member's cells are ordered
// on their own), so the members of a warp's cells are non-decreasing in lane
// order.
#pragma once
#include <cmath>
#include <cstdint>

#include "hg_state.hpp"

namespace hg {

// Member of cell c (c < memberOff[nMembers]): one coalesced load of the
// per-cell table (a binary search over the members' offsets took eight
// dependent loads per cell and stage).
__device__ __forceinline__ int member_of(const DevScalars& s, int c) { return __ldg(&s.memberOfCell[c]); }

// Min of v over the lanes of the warp with the same member m (m
// non-decreasing in lane order; every lane takes part); the first lane of each
// member's run publishes it with one atomicMin on the IEEE bits (non-negative
// values order like unsigned integers), so the result does not depend on
// the order the warps finish in.
__device__ __forceinline__ void member_min_publish_f(const DevScalars& s, float v, int m) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float vo = __shfl_down_sync(0xffffffffu, v, o);
    const int mo = __shfl_down_sync(0xffffffffu, m, o);
    if (lane + o < 32 && mo == m) v = fminf(v, vo);
  }
  const int mp = __shfl_up_sync(0xffffffffu, m, 1);
  if ((lane == 0 || mp != m) && m >= 0 && v < INFINITY) atomicMin(&s.cflMinMF[m], __float_as_uint(v));
}

__device__ __forceinline__ void member_min_publish(const DevScalars& s, double v, int m) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double vo = __shfl_down_sync(0xffffffffu, v, o);
    const int mo = __shfl_down_sync(0xffffffffu, m, o);
    if (lane + o < 32 && mo == m) v = fmin(v, vo);
  }
  const int mp = __shfl_up_sync(0xffffffffu, m, 1);
  if ((lane == 0 || mp != m) && m >= 0 && v < INFINITY)
    atomicMin(&s.cflMinM[m], (unsigned long long)__double_as_longlong(v));
}

}  // namespace hg
