// State-dependent flow resistance: the per-cell Manning n (or the friction
// magnitude of the flow-resistance closure) recomputed from each RHS
// evaluation's input state, before the inlet-Q conveyance totals and the stage
// kernel read it.
//
//  * n(h, Umag, ks) functions: process_ManningN_2D.jl:140-213, evaluated on the
//    clamped state with Umag = |q| / h (semi_discretize_swe_2D.jl:101-106,141-149).
//  * UDE closures: process_ManningN_2D.jl:216-273 (n from the network) and
//    process_FlowResistance_UDE.jl:3-45 (friction magnitude from the network),
//    the network being process_UDE.jl:3-56's Lux chain: per hidden layer
//    Dense(in, w, act) then LayerNorm(w); a linear Dense(w, 1); the output
//    bound lo + (hi - lo) sigmoid(y).  LayerNorm takes its statistics over the
//    whole (width x cells) batch, as Lux's LayerNorm does with its default
//    dims = Colon(), so each hidden layer needs two reductions over all cells
//    (mean, then the uncorrected variance about it) before the next layer can
//    be evaluated; with overBatch = 0 the statistics are each cell's own.
//
// FP64 kernels round as the oracle does (no FMA in this file); the FP32 kernels
// serve the FP32-compensated path and read its hi/lo state records.
#include <cmath>

#include "hg_device.cuh"
#include "hg_f32.cuh"
#include "hg_reduce.cuh"
#include "hg_resfn.cuh"
#include "hg_state.hpp"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = 256;

// NNlib's sigmoid (exp of -|x|, no overflow).
template <class S>
__device__ __forceinline__ S sigmoid_nn(S x) {
  const S t = RM<S>::exp(-RM<S>::abs(x));
  return x >= S(0) ? S(1) / (S(1) + t) : t / (S(1) + t);
}

template <class S>
__device__ __forceinline__ S activation(int a, S x) {
  switch (a) {
    case 0: return x > S(0) ? x : S(0);                      // relu
    case 1: return x > S(0) ? x : S(0.01) * x;               // leakyrelu
    case 2: return sigmoid_nn(x);
    case 3: return RM<S>::tanh(x);
    default: return RM<S>::log1p(RM<S>::exp(-RM<S>::abs(x))) + (x > S(0) ? x : S(0));   // softplus
  }
}

template <class S>
__device__ __forceinline__ S normalise(S x, double lo, double hi) {
  return S(2.0) * (x - S(lo)) / (S(hi) - S(lo)) - S(1.0);
}

// Clamped state of cell c (semi_discretize_swe_2D.jl:101-106).
__device__ __forceinline__ void cell_state(const DevMesh& m, const double* __restrict__ Q, int c, double& h,
                                           double& qx, double& qy) {
  const double d = Q[c] + m.hst[c];
  const bool dry = d <= m.hsm;
  h = dry ? m.hsm : d;
  qx = dry ? 0.0 : Q[m.n + c];
  qy = dry ? 0.0 : Q[2 * m.n + c];
}
__device__ __forceinline__ void cell_state(const DevMesh& m, StateF32 X, int c, float& h, float& qx, float& qy) {
  const SideF32 L = make_side_f32(X.x[c], m.CP[c], m.hsmf, m.hsmLo);
  h = L.s.h;
  qx = L.s.hu;
  qy = L.s.hv;
}

// Network inputs of one cell (process_ManningN_2D.jl:228-236; process_FlowResistance_UDE.jl:13-20).
template <class S>
__device__ __forceinline__ void ude_inputs(const ResDev& r, int c, S h, S qx, S qy, S (&a)[kResMaxWidth]) {
#pragma unroll
  for (int i = 0; i < kResMaxWidth; ++i) a[i] = S(0);
  a[0] = normalise(h, r.lo[0], r.hi[0]);
  if (r.kind == kResUdeManningHUmagKs) {
    const S u = qx / h, v = qy / h;
    a[1] = normalise(RM<S>::sqrt(u * u + v * v), r.lo[1], r.hi[1]);
    a[2] = normalise(S(r.ks[c]), r.lo[2], r.hi[2]);
  } else if (r.kind == kResUdeFlowResistance) {   // q bounds = h bounds x velocity-magnitude bounds
    a[1] = normalise(smooth_sqrt(qx * qx + qy * qy), r.lo[0] * r.lo[1], r.hi[0] * r.hi[1]);
  }
}

// z = act(W a + b) of one Dense layer (weights at offset off, out x din column-major).
template <class S>
__device__ __forceinline__ void dense_act(const ResDev& r, int off, int din, int w, int act, const S (&a)[kResMaxWidth],
                                          S (&z)[kResMaxWidth]) {
#pragma unroll
  for (int o = 0; o < kResMaxWidth; ++o) {
    S s = S(0);
    if (o < w) {
#pragma unroll
      for (int i = 0; i < kResMaxWidth; ++i)
        if (i < din) s += RM<S>::w(r, off + o + i * w) * a[i];
      s = activation(act, s + RM<S>::w(r, off + w * din + o));
    }
    z[o] = s;
  }
}

// a = LayerNorm(z) with the statistics of layer l.
template <class S>
__device__ __forceinline__ void layer_norm(const ResDev& r, int off, int w, int l, const S (&z)[kResMaxWidth],
                                           S (&a)[kResMaxWidth]) {
  S mu, var;
  if (r.overBatch) {
    mu = S(r.stats[2 * l]);
    var = S(r.stats[2 * l + 1]);
  } else {
    S s = S(0), q = S(0);
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o)
      if (o < w) s += z[o];
    mu = s / S(w);
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o)
      if (o < w) q += (z[o] - mu) * (z[o] - mu);
    var = q / S(w);
  }
  const S den = RM<S>::sqrt(var + S(r.lnEps));
#pragma unroll
  for (int o = 0; o < kResMaxWidth; ++o)
    a[o] = o < w ? (z[o] - mu) / den * RM<S>::w(r, off + o) + RM<S>::w(r, off + w + o) : S(0);
}

// Runs hidden layers [0, upto) on a; leaves in z the post-activation values of
// layer `upto` when upto < nHidden.  Returns the parameter offset reached and
// the width of a.
template <class S>
__device__ __forceinline__ int mlp_run(const ResDev& r, int upto, S (&a)[kResMaxWidth], S (&z)[kResMaxWidth], int& din) {
  int off = 0;
  din = r.inDim;
  for (int l = 0; l < r.nHidden; ++l) {
    const int w = r.width[l];
    dense_act(r, off, din, w, r.act[l], a, z);
    off += w * din + w;
    if (l == upto) return off;
    layer_norm(r, off, w, l, z, a);
    off += 2 * w;
    din = w;
  }
  return off;
}

template <class S>
__device__ __forceinline__ S mlp_output(const ResDev& r, int off, int din, const S (&a)[kResMaxWidth]) {
  S s = S(0);
#pragma unroll
  for (int i = 0; i < kResMaxWidth; ++i)
    if (i < din) s += RM<S>::w(r, off + i) * a[i];
  return S(r.outLo) + (S(r.outHi) - S(r.outLo)) * sigmoid_nn(s + RM<S>::w(r, off + din));
}

// One LayerNorm statistics pass over all cells: which = 0 sums layer l's
// post-activation values (-> mean), which = 1 their squared deviations from
// that mean (-> uncorrected variance).  Per-block partials; the last block adds
// them in block order (deterministic) and stores stats[2 l + which].
template <class S, class State>
__global__ void __launch_bounds__(kBlock) k_res_stats(DevMesh m, State Q, int l, int which) {
  const ResDev& r = m.res;
  const int w = r.width[l];
  const S mu = which ? S(r.stats[2 * l]) : S(0);
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.n; c += gridDim.x * blockDim.x) {
    S h, qx, qy;
    cell_state(m, Q, c, h, qx, qy);
    S a[kResMaxWidth], z[kResMaxWidth];
    ude_inputs(r, c, h, qx, qy, a);
    int din;
    mlp_run(r, l, a, z, din);
    S s = S(0);
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o)
      if (o < w) s += which ? (z[o] - mu) * (z[o] - mu) : z[o];
    acc += (double)s;
  }
  const double b = block_sum(acc);
  __shared__ int isLast;
  if (threadIdx.x == 0) {
    r.partials[blockIdx.x] = b;
    __threadfence();
    isLast = (atomicAdd(r.ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!isLast) return;
  __threadfence();
  double s = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) s += __ldcg(&r.partials[k]);
  const double tot = block_sum(s);
  if (threadIdx.x == 0) {
    r.stats[2 * l + which] = tot / ((double)m.n * (double)w);
    *r.ticket = 0u;
  }
}

// The per-cell resistance of the state.
template <class S, class State>
__global__ void __launch_bounds__(kBlock) k_res_cells(DevMesh m, State Q) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const ResDev& r = m.res;
  S h, qx, qy;
  cell_state(m, Q, c, h, qx, qy);
  S out;
  if (r.kind <= kResHUmagKs) {
    const S u = qx / h, v = qy / h;
    out = manning_fn(r, h, RM<S>::sqrt(u * u + v * v), r.ks ? S(r.ks[c]) : S(0));
  } else {
    S a[kResMaxWidth], z[kResMaxWidth];
    ude_inputs(r, c, h, qx, qy, a);
    int din;
    const int off = mlp_run(r, r.nHidden, a, z, din);
    out = mlp_output(r, off, din, a);
  }
  if constexpr (sizeof(S) == 8) {
    if (r.kind == kResUdeFlowResistance) r.fres[c] = out;
    else const_cast<double*>(m.man)[c] = out;
  } else {
    if (r.kind == kResUdeFlowResistance) r.fresF[c] = out;
    else reinterpret_cast<float*>(const_cast<float4*>(m.CP) + c)[3] = out;   // CP.w
  }
}

template <class S, class State>
int launch_resistance(const DevMesh& m, State Q, cudaStream_t st) {
  if (m.res.kind == kResConstant || m.n == 0) return 0;
  int launches = 0;
  if (m.res.kind >= kResUdeManningH && m.res.overBatch) {
    const int64_t b = (m.n + kBlock - 1) / kBlock;
    const int grid = (int)(b < kResPartials ? b : kResPartials);
    for (int l = 0; l < m.res.nHidden; ++l)
      for (int which = 0; which < 2; ++which) {
        k_res_stats<S, State><<<grid, kBlock, 0, st>>>(m, Q, l, which);
        ++launches;
      }
  }
  k_res_cells<S, State><<<(m.n + kBlock - 1) / kBlock, kBlock, 0, st>>>(m, Q);
  return launches + 1;
}

}  // namespace

int resistance_launches(const DevMesh& m) {
  if (m.res.kind == kResConstant || m.n == 0) return 0;
  return 1 + ((m.res.kind >= kResUdeManningH && m.res.overBatch) ? 2 * m.res.nHidden : 0);
}

int launch_resistance_f64(const DevMesh& m, const double* Q, cudaStream_t st) {
  return launch_resistance<double, const double*>(m, Q, st);
}

int launch_resistance_f32(const DevMesh& m, StateF32 X, cudaStream_t st) {
  return launch_resistance<float, StateF32>(m, X, st);
}

}  // namespace hg
