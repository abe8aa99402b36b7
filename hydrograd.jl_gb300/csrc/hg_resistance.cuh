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
// The kernels are templates, instantiated by two translation units:
// hg_resistance.cu (FP64, compiled without FMA contraction so that it rounds
// as the oracle does) and hg_resistance_f32.cu (FP32, for the
// FP32-compensated path, reading its hi/lo state records; FMA contraction on).
#pragma once
#include <cmath>

#include "hg_adjoint_state.hpp"
#include "hg_device.cuh"
#include "hg_f32.cuh"
#include "hg_reduce.cuh"
#include "hg_resfn.cuh"
#include "hg_state.hpp"

namespace hg {

using namespace hgd;
using namespace devred;

namespace {

constexpr int kBlock = kResBlock;

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
// ACT >= 0: the activation fixed at compile time; ACT < 0: a, at run time.
template <int ACT, class S>
__device__ __forceinline__ S activation_as(int a, S x) {
  return activation(ACT >= 0 ? ACT : a, x);
}

template <class S>
__device__ __forceinline__ S normalise(S x, S lo, S hi) {
  return S(2.0) * (x - lo) / (hi - lo) - S(1.0);
}

// The network's input bounds and output bound in the kernel's precision,
// converted once per thread (a double-to-float conversion runs on the FP64
// pipe).
template <class S>
struct NetConsts {
  S lo[kResMaxInputs], hi[kResMaxInputs];
  S qlo, qhi;   // the flow-resistance closure's discharge bounds (h bounds x velocity-magnitude bounds)
  S outLo, outHi;
};
template <class S>
__device__ __forceinline__ NetConsts<S> net_consts(const ResDev& r) {
  NetConsts<S> k;
#pragma unroll
  for (int i = 0; i < kResMaxInputs; ++i) {
    k.lo[i] = S(r.lo[i]);
    k.hi[i] = S(r.hi[i]);
  }
  k.qlo = S(r.lo[0] * r.lo[1]);
  k.qhi = S(r.hi[0] * r.hi[1]);
  k.outLo = S(r.outLo);
  k.outHi = S(r.outHi);
  return k;
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

__device__ __forceinline__ bool cell_dry(const DevMesh& m, const double* __restrict__ Q, int c) {
  return Q[c] + m.hst[c] <= m.hsm;
}
__device__ __forceinline__ bool cell_dry(const DevMesh& m, StateF32 X, int c) {
  return make_side_f32(X.x[c], m.CP[c], m.hsmf, m.hsmLo).s.dry;
}

// Network inputs of one cell (process_ManningN_2D.jl:228-236; process_FlowResistance_UDE.jl:13-20).
// (MW: the register arrays' length, a bound on the widths; the forward kernels
// take the smallest of 4, 8, 16 that holds the network.)
template <class S, int MW>
__device__ __forceinline__ void ude_inputs(const ResDev& r, const NetConsts<S>& k, int c, S h, S qx, S qy,
                                           S (&a)[MW]) {
  static_assert(MW >= kResMaxInputs, "the inputs need kResMaxInputs values");
#pragma unroll
  for (int i = 0; i < MW; ++i) a[i] = S(0);
  a[0] = normalise(h, k.lo[0], k.hi[0]);
  if (r.kind == kResUdeManningHUmagKs) {
    const S u = qx / h, v = qy / h;
    a[1] = normalise(RM<S>::sqrt(u * u + v * v), k.lo[1], k.hi[1]);
    a[2] = normalise(S(r.ks[c]), k.lo[2], k.hi[2]);
  } else if (r.kind == kResUdeFlowResistance) {
    a[1] = normalise(smooth_sqrt(qx * qx + qy * qy), k.qlo, k.qhi);
  }
}
template <class S, int MW>
__device__ __forceinline__ void ude_inputs(const ResDev& r, int c, S h, S qx, S qy, S (&a)[MW]) {
  ude_inputs(r, net_consts<S>(r), c, h, qx, qy, a);
}

// z = act(W a + b) of one Dense layer (weights at offset off, out x din column-major).
template <class S, int MW>
__device__ __forceinline__ void dense_act(const ResDev& r, int off, int din, int w, int act, const S (&a)[MW],
                                          S (&z)[MW]) {
#pragma unroll
  for (int o = 0; o < MW; ++o) {
    S s = S(0);
    if (o < w) {
#pragma unroll
      for (int i = 0; i < MW; ++i)
        if (i < din) s += RM<S>::w(r, off + o + i * w) * a[i];
      s = activation(act, s + RM<S>::w(r, off + w * din + o));
    }
    z[o] = s;
  }
}

// a = LayerNorm(z) with the statistics of layer l.
template <class S, int MW>
__device__ __forceinline__ void layer_norm(const ResDev& r, int off, int w, int l, const S (&z)[MW], S (&a)[MW]) {
  S mu, var;
  if (r.overBatch) {
    mu = S(r.stats[2 * l]);
    var = S(r.stats[2 * l + 1]);
  } else {
    S s = S(0), q = S(0);
#pragma unroll
    for (int o = 0; o < MW; ++o)
      if (o < w) s += z[o];
    mu = s / S(w);
#pragma unroll
    for (int o = 0; o < MW; ++o)
      if (o < w) q += (z[o] - mu) * (z[o] - mu);
    var = q / S(w);
  }
  const S den = RM<S>::sqrt(var + S(r.lnEps));
#pragma unroll
  for (int o = 0; o < MW; ++o)
    a[o] = o < w ? (z[o] - mu) / den * RM<S>::w(r, off + o) + RM<S>::w(r, off + w + o) : S(0);
}

// Runs hidden layers [0, upto) on a; leaves in z the post-activation values of
// layer `upto` when upto < nHidden.  Returns the parameter offset reached and
// the width of a.
template <class S, int MW>
__device__ __forceinline__ int mlp_run(const ResDev& r, int upto, S (&a)[MW], S (&z)[MW], int& din) {
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

template <class S, int MW>
__device__ __forceinline__ S mlp_output(const ResDev& r, int off, int din, const S (&a)[MW]) {
  S s = S(0);
#pragma unroll
  for (int i = 0; i < MW; ++i)
    if (i < din) s += RM<S>::w(r, off + i) * a[i];
  return S(r.outLo) + (S(r.outHi) - S(r.outLo)) * sigmoid_nn(s + RM<S>::w(r, off + din));
}

// Parameter offset of hidden layer l's Dense weights, and that layer's input
// width; the first cache row of layer l.
__device__ __forceinline__ int layer_offset(const ResDev& r, int l, int& din) {
  int off = 0;
  din = r.inDim;
  for (int k = 0; k < l; ++k) {
    off += r.width[k] * din + 3 * r.width[k];
    din = r.width[k];
  }
  return off;
}
__device__ __forceinline__ int hidden_row(const ResDev& r, int l) {
  int row = 0;
  for (int k = 0; k < l; ++k) row += r.width[k];
  return row;
}

// Layer l's post-activation values of cell c from the cache.
template <class S, int MW>
__device__ __forceinline__ void load_hidden(const ResDev& r, int l, int n, int c, S (&z)[MW]) {
  const S* __restrict__ hid = RM<S>::hid(r) + (size_t)hidden_row(r, l) * n + c;
  const int w = r.width[l];
#pragma unroll
  for (int o = 0; o < MW; ++o) z[o] = o < w ? hid[(size_t)o * n] : S(0);
}

// One layer's parameters in shared memory, padded to MW x MW so that the
// unrolled loops address them at constant offsets: W[i][o] (input i, output
// o), the bias, and the LayerNorm scale and bias applied to the layer's input
// (the layer before's normalisation; zero where there is none).
template <class S, int MW>
struct LayerParams {
  S W[MW][MW];
  S b[MW];
  S g[MW], be[MW];
};

// Stages the Dense layer at parameter offset off (din -> w) and the LayerNorm
// at lnOff (scale then bias, din each; lnOff < 0: none).  All threads of the
// block take part.
template <class S, int MW>
__device__ __forceinline__ void stage_params(const ResDev& r, int off, int din, int w, int lnOff,
                                             LayerParams<S, MW>& P) {
  for (int k = threadIdx.x; k < MW * MW; k += blockDim.x) {
    const int i = k / MW, o = k % MW;
    P.W[i][o] = (i < din && o < w) ? RM<S>::w(r, off + o + i * w) : S(0);
  }
  for (int o = threadIdx.x; o < MW; o += blockDim.x) {
    P.b[o] = o < w ? RM<S>::w(r, off + w * din + o) : S(0);
    P.g[o] = (lnOff >= 0 && o < din) ? RM<S>::w(r, lnOff + o) : S(0);
    P.be[o] = (lnOff >= 0 && o < din) ? RM<S>::w(r, lnOff + din + o) : S(0);
  }
  __syncthreads();
}

// a = LayerNorm(z) over w values with the batch statistics (mu, den) and the
// staged scale and bias.  FP64 divides by den as the oracle does; FP32
// multiplies by its reciprocal (den is the same for every cell).
template <class S, int MW>
__device__ __forceinline__ void layer_norm_staged(const LayerParams<S, MW>& P, int w, S mu, S den, const S (&z)[MW],
                                                  S (&a)[MW]) {
  if constexpr (sizeof(S) == 4) {
    const S rden = S(1) / den;
#pragma unroll
    for (int o = 0; o < MW; ++o) a[o] = o < w ? (z[o] - mu) * rden * P.g[o] + P.be[o] : S(0);
  } else {
#pragma unroll
    for (int o = 0; o < MW; ++o) a[o] = o < w ? (z[o] - mu) / den * P.g[o] + P.be[o] : S(0);
  }
}

// Batch statistics of hidden layer l: mean and LayerNorm denominator.
template <class S>
__device__ __forceinline__ void batch_stats(const ResDev& r, int l, S& mu, S& den) {
  mu = S(r.stats[2 * l]);
  den = RM<S>::sqrt(S(r.stats[2 * l + 1]) + S(r.lnEps));
}

// z = act(W a + b) with the staged Dense layer; each output's terms are added
// in input order, then the bias, as dense_act does.
template <int ACT, class S, int MW>
__device__ __forceinline__ void dense_act_staged(const LayerParams<S, MW>& P, int din, int w, int act,
                                                 const S (&a)[MW], S (&z)[MW]) {
  S s[MW];
#pragma unroll
  for (int o = 0; o < MW; ++o) s[o] = S(0);
#pragma unroll
  for (int i = 0; i < MW; ++i)
    if (i < din) {
#pragma unroll
      for (int o = 0; o < MW; ++o) s[o] += P.W[i][o] * a[i];
    }
#pragma unroll
  for (int o = 0; o < MW; ++o) z[o] = o < w ? activation_as<ACT>(act, s[o] + P.b[o]) : S(0);
}

template <class S>
__device__ __forceinline__ double block_total(S v) {
  if constexpr (sizeof(S) == 4) return block_sum_f32(v);
  else return block_sum(v);
}

// LayerNorm over the batch, hidden layer l.  Each thread takes cells
// c = start + k stride (a grid of one wave; the block's parameters staged
// once): the layer evaluated from the inputs, or from layer l - 1's cached
// values normalised with its statistics, and its post-activation values
// cached.  Its mean and uncorrected variance over all (cells x w) values in
// the same launch: each block its sum S_b, then its mean m_b and the squared
// deviations about it M2_b (the block's own cached values read back, from
// L2); the last block combines the blocks' in block order (deterministic) by
// Chan, Golub and LeVeque's pairwise update: mean = sum S_b / N,
// M2 = sum (M2_b + N_b (m_b - mean)^2) -- the two-pass variance with one pass
// over the layer's inputs.
template <class S, class State, int MW, int ACT>
__global__ void __launch_bounds__(kBlock) k_res_layer(DevMesh m, State Q, int l) {
  const ResDev& r = m.res;
  __shared__ LayerParams<S, MW> P;
  __shared__ double sMean;
  __shared__ int isLast;
  const int w = r.width[l];
  int din;
  const int off = layer_offset(r, l, din);
  stage_params(r, off, din, w, l > 0 ? off - 2 * din : -1, P);
  S mu = S(0), den = S(1);
  if (l > 0) batch_stats(r, l - 1, mu, den);
  const NetConsts<S> nk = net_consts<S>(r);
  const int n = m.n, stride = gridDim.x * blockDim.x;
  S* __restrict__ hid = RM<S>::hid(r) + (size_t)hidden_row(r, l) * n;
  S sum = S(0);
  int cells = 0;   // this thread's
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride) {
    S a[MW], z[MW];
    if (l == 0) {
      S h, qx, qy;
      cell_state(m, Q, c, h, qx, qy);
      ude_inputs(r, nk, c, h, qx, qy, a);
    } else {
      S zp[MW];
      load_hidden(r, l - 1, n, c, zp);
      layer_norm_staged(P, din, mu, den, zp, a);
    }
    dense_act_staged<ACT>(P, din, w, r.act[l], a, z);
#pragma unroll
    for (int o = 0; o < MW; ++o)
      if (o < w) {
        hid[(size_t)o * n + c] = z[o];
        sum += z[o];
      }
    ++cells;
  }
  const double Sb = block_total(sum);
  const double Nb = (double)block_total(S(cells)) * (double)w;
  if (threadIdx.x == 0) sMean = Nb > 0.0 ? Sb / Nb : 0.0;
  __syncthreads();
  const double mb = sMean;
  const S cb = S(mb);   // the deviations' centre in the kernel's precision
  S q = S(0);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride) {
#pragma unroll
    for (int o = 0; o < MW; ++o)
      if (o < w) {
        const S d = hid[(size_t)o * n + c] - cb;
        q += d * d;
      }
  }
  const double Qb = block_total(q);
  if (threadIdx.x == 0) {
    const double d = mb - (double)cb;   // about m_b: sum (z - c)^2 - N_b (m_b - c)^2
    double* pb = r.partials + 4 * (size_t)blockIdx.x;
    pb[0] = Sb;
    pb[1] = Qb - Nb * d * d;
    pb[2] = Nb;
    pb[3] = mb;
    __threadfence();
    isLast = (atomicAdd(r.ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!isLast) return;
  __threadfence();
  const double N = (double)n * (double)w;
  double t = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) t += __ldcg(&r.partials[4 * (size_t)k]);
  const double tot = block_sum(t);
  if (threadIdx.x == 0) sMean = tot / N;
  __syncthreads();
  const double mean = sMean;
  double u = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    const double* pk = r.partials + 4 * (size_t)k;
    const double dk = __ldcg(&pk[3]) - mean;
    u += __ldcg(&pk[1]) + __ldcg(&pk[2]) * dk * dk;
  }
  const double M2 = block_sum(u);
  if (threadIdx.x == 0) {
    r.stats[2 * l] = mean;
    r.stats[2 * l + 1] = M2 / N;
    *r.ticket = 0u;
  }
}

// The per-cell resistance of the state (grid-stride), by PATH: kPathFn an
// n(h, Umag, ks) function; kPathCached the network's last hidden layer from
// the LayerNorm-over-the-batch cache, normalised, then its output layer
// (staged once a block); kPathNet the whole network per cell.
constexpr int kPathFn = 0, kPathCached = 1, kPathNet = 2;
template <class S, class State, int MW, int PATH>
__global__ void __launch_bounds__(kBlock) k_res_cells(DevMesh m, State Q) {
  const ResDev& r = m.res;
  constexpr bool cached = PATH == kPathCached;
  __shared__ LayerParams<S, MW> P;   // the output layer and the last hidden layer's LayerNorm
  int din = 0;
  S mu = S(0), den = S(1);
  const NetConsts<S> nk = net_consts<S>(r);
  if constexpr (cached) {
    const int offOut = layer_offset(r, r.nHidden, din);
    stage_params(r, offOut, din, 1, offOut - 2 * din, P);
    batch_stats(r, r.nHidden - 1, mu, den);
  }
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.n; c += gridDim.x * blockDim.x) {
    S h, qx, qy;
    cell_state(m, Q, c, h, qx, qy);
    S out;
    if constexpr (PATH == kPathFn) {
      const S u = qx / h, v = qy / h;
      out = manning_fn(r, h, RM<S>::sqrt(u * u + v * v), r.ks ? S(r.ks[c]) : S(0));
    } else if constexpr (cached) {
      S a[MW], z[MW];
      load_hidden(r, r.nHidden - 1, m.n, c, z);
      layer_norm_staged(P, din, mu, den, z, a);
      S t = S(0);
#pragma unroll
      for (int i = 0; i < MW; ++i)
        if (i < din) t += P.W[i][0] * a[i];
      out = nk.outLo + (nk.outHi - nk.outLo) * sigmoid_nn(t + P.b[0]);
    } else {
      S a[MW], z[MW];
      int dl;
      ude_inputs(r, nk, c, h, qx, qy, a);
      const int off = mlp_run(r, r.nHidden, a, z, dl);
      out = mlp_output(r, off, dl, a);
    }
    if constexpr (sizeof(S) == 8) {
      if (r.kind == kResUdeFlowResistance) r.fres[c] = out;
      else const_cast<double*>(m.man)[c] = out;
    } else {
      if (r.kind == kResUdeFlowResistance) r.fresF[c] = out;
      else reinterpret_cast<float*>(const_cast<float4*>(m.CP) + c)[3] = out;   // CP.w
    }
  }
}

// One wave: the SMs times the blocks of kernel k resident on one.
template <class K>
int one_wave(K k, int64_t blocksNeeded) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, kBlock, 0);
  const int64_t g = (int64_t)(sms > 0 ? sms : 1) * (per > 0 ? per : 1);
  return (int)(blocksNeeded < g ? blocksNeeded : g);
}

template <class S, class State, int MW, int PATH>
void launch_cells(const DevMesh& m, State Q, cudaStream_t st) {
  static const int g = one_wave(k_res_cells<S, State, MW, PATH>, 1 << 30);
  const int64_t need = res_stat_blocks(m.n);
  k_res_cells<S, State, MW, PATH><<<(int)(need < g ? need : g), kBlock, 0, st>>>(m, Q);
}

template <class S, class State, int MW, int ACT>
void launch_layer(const DevMesh& m, State Q, int l, cudaStream_t st) {
  static const int g = one_wave(k_res_layer<S, State, MW, ACT>, 1 << 30);
  const int64_t need = res_stat_blocks(m.n);
  k_res_layer<S, State, MW, ACT><<<(int)(need < g ? need : g), kBlock, 0, st>>>(m, Q, l);
}

template <class S, class State, int MW>
int launch_resistance_w(const DevMesh& m, State Q, cudaStream_t st) {
  const ResDev& r = m.res;
  if (r.kind <= kResHUmagKs) {
    launch_cells<S, State, MW, kPathFn>(m, Q, st);
    return 1;
  }
  if (!r.overBatch || r.nHidden == 0) {
    launch_cells<S, State, MW, kPathNet>(m, Q, st);
    return 1;
  }
  for (int l = 0; l < r.nHidden; ++l) {
    if constexpr (sizeof(S) == 4) {   // the activation a template argument (FP64: read at run time)
      switch (r.act[l]) {
        case 0: launch_layer<S, State, MW, 0>(m, Q, l, st); break;
        case 1: launch_layer<S, State, MW, 1>(m, Q, l, st); break;
        case 2: launch_layer<S, State, MW, 2>(m, Q, l, st); break;
        case 3: launch_layer<S, State, MW, 3>(m, Q, l, st); break;
        default: launch_layer<S, State, MW, 4>(m, Q, l, st); break;
      }
    } else {
      launch_layer<S, State, MW, -1>(m, Q, l, st);
    }
  }
  launch_cells<S, State, MW, kPathCached>(m, Q, st);
  return r.nHidden + 1;
}

template <class S, class State>
int launch_resistance(const DevMesh& m, State Q, cudaStream_t st) {
  if (m.res.kind == kResConstant || m.n == 0) return 0;
  int wmax = 0;
  if (m.res.kind >= kResUdeManningH)
    for (int l = 0; l < m.res.nHidden; ++l) wmax = m.res.width[l] > wmax ? m.res.width[l] : wmax;
  if (wmax <= 4) return launch_resistance_w<S, State, 4>(m, Q, st);
  if (wmax <= 8) return launch_resistance_w<S, State, 8>(m, Q, st);
  return launch_resistance_w<S, State, kResMaxWidth>(m, Q, st);
}

// ---------------------------------------------------------------------------
// VJP of the UDE network (the closure's Lux chain differentiated as Zygote
// does through swe_2D_UDE.jl:119,522's loss): reverse mode per cell, from the
// stage's cotangent g = beta dL/dy of the network output y (n, or F of the
// flow-resistance closure) back to the cell's inputs and to the parameters.
//   y = lo + (hi - lo) s(t), t = w . a^H + b:    dt = g (hi - lo) s (1 - s)
//   a^(l+1) = gamma xh + beta, xh = (z - mu) / den, den = sqrt(var + eps):
//     dgamma += da xh, dbeta += da, dxh = da gamma,
//     dz = (dxh - mean(dxh) - xh mean(dxh xh)) / den
//   (the means over the cell's own w values, or -- LayerNorm over the batch --
//   over all cells' w values, which makes each hidden layer one more pass:
//   the sums of dxh and dxh xh over all cells are needed before the layer's
//   dz, and they need the layers above already taken back);
//   z = act(p), p = W a + b: dp = dz act'(p), dW += dp a^T, db += dp, da = W^T dp.
// Each thread takes one cell per round (a warp, 32 cells); the parameter
// terms of the round are staged in shared memory and summed over the 32
// cells by the lane owning the parameter, into per-block sums; the last block
// adds the blocks' sums in block order into gTheta.  Fixed grid, fixed order:
// the sums are reproducible run to run.

constexpr int kUdeRow = kResMaxWidth + 1;                         // padded staging rows
constexpr int kUdeMaxParams = (kResMaxWidth * kResMaxInputs + 3 * kResMaxWidth) +
                              (kResMaxLayers - 1) * (kResMaxWidth * kResMaxWidth + 3 * kResMaxWidth) +
                              kResMaxWidth + 1;

template <class S>
__device__ __forceinline__ S activation_grad(int a, S p, S z) {
  switch (a) {
    case 0: return p > S(0) ? S(1) : S(0);          // relu
    case 1: return p > S(0) ? S(1) : S(0.01);       // leakyrelu
    case 2: return z * (S(1) - z);                  // sigmoid
    case 3: return S(1) - z * z;                    // tanh
    default: return sigmoid_nn(p);                  // softplus
  }
}

// One hidden layer of one cell: pre-activations, post-activations, the
// normalised values and the LayerNorm denominator.
template <class S>
struct UdeLayer {
  S p[kResMaxWidth], z[kResMaxWidth], xh[kResMaxWidth];
  S den;
};

// Forward from the inputs a to hidden layer `target`; leaves in a that
// layer's input (width din) and in L its values.  Returns its parameter offset.
template <class S>
__device__ __forceinline__ int ude_forward_to(const ResDev& r, int target, S (&a)[kResMaxWidth], UdeLayer<S>& L,
                                              int& din) {
  int off = 0;
  din = r.inDim;
  for (int l = 0;; ++l) {
    const int w = r.width[l];
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o) {
      S s = S(0);
      if (o < w) {
#pragma unroll
        for (int i = 0; i < kResMaxWidth; ++i)
          if (i < din) s += RM<S>::w(r, off + o + i * w) * a[i];
        s = s + RM<S>::w(r, off + w * din + o);
      }
      L.p[o] = s;
      L.z[o] = o < w ? activation(r.act[l], s) : S(0);
    }
    S mu, var;
    if (r.overBatch) {
      mu = S(r.stats[2 * l]);
      var = S(r.stats[2 * l + 1]);
    } else {
      S s = S(0), q = S(0);
#pragma unroll
      for (int o = 0; o < kResMaxWidth; ++o)
        if (o < w) s += L.z[o];
      mu = s / S(w);
#pragma unroll
      for (int o = 0; o < kResMaxWidth; ++o)
        if (o < w) q += (L.z[o] - mu) * (L.z[o] - mu);
      var = q / S(w);
    }
    L.den = RM<S>::sqrt(var + S(r.lnEps));
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o) L.xh[o] = o < w ? (L.z[o] - mu) / L.den : S(0);
    if (l == target) return off;
    off += w * din + w;
#pragma unroll
    for (int o = 0; o < kResMaxWidth; ++o)
      a[o] = o < w ? L.xh[o] * RM<S>::w(r, off + o) + RM<S>::w(r, off + w + o) : S(0);
    off += 2 * w;
    din = w;
  }
}

// Warp sum in a fixed tree (every lane gets the total).
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// pass >= 0 (LayerNorm over the batch only): the sums over all cells of
// layer `pass`'s dxh and dxh xh, into a.udeS[2 pass], a.udeS[2 pass + 1]
// (the layers above taken back with their sums from earlier passes).
// pass < 0: the whole VJP -- the state cotangents into out, the parameters
// into gTheta.
template <class S, class State, class Out>
__global__ void __launch_bounds__(32) k_ude_vjp(DevMesh m, AdjDev ad, State Q, Out* out, int pass) {
  const ResDev& r = m.res;
  const int H = r.nHidden, n = m.n, P = ad.udeP, lane = threadIdx.x;
  const bool fin = pass < 0;
  __shared__ S sA[32][kUdeRow], sG[32][kUdeRow], sX[32][kUdeRow], sD[32][kUdeRow];
  __shared__ double sAcc[kUdeMaxParams];
  if (fin)
    for (int p = lane; p < P; p += 32) sAcc[p] = 0.0;
  double s1 = 0.0, s2 = 0.0;
  // The parameter sums of one round: nl parameters from offset off; term(k, p)
  // reads the staged values of the round's cell k.
  auto reduce = [&](int off, int nl, auto term) {
    __syncwarp();
    for (int p = lane; p < nl; p += 32) {
      double t = 0.0;
      for (int k = 0; k < 32; ++k) t += (double)term(k, p);
      sAcc[off + p] += t;
    }
    __syncwarp();
  };
  for (int base = blockIdx.x * 32; base < n; base += gridDim.x * 32) {
    const int c = base + lane;
    const bool live = c < n;
    const int cc = live ? c : 0;
    S h, qx, qy;
    cell_state(m, Q, cc, h, qx, qy);
    const S g = live ? S(ad.udeGn[cc]) : S(0);
    if (!r.overBatch && __all_sync(0xffffffffu, g == S(0))) continue;   // the round adds nothing
    // output layer
    S a[kResMaxWidth], z[kResMaxWidth];
    ude_inputs(r, cc, h, qx, qy, a);
    int din;
    const int offOut = mlp_run(r, H, a, z, din);
    S t = S(0);
#pragma unroll
    for (int i = 0; i < kResMaxWidth; ++i)
      if (i < din) t += RM<S>::w(r, offOut + i) * a[i];
    const S sg = sigmoid_nn(t + RM<S>::w(r, offOut + din));
    const S dt = g * (S(r.outHi) - S(r.outLo)) * sg * (S(1) - sg);
    if (fin) {
#pragma unroll
      for (int i = 0; i < kResMaxWidth; ++i) sA[lane][i] = a[i];
      sG[lane][0] = dt;
      reduce(offOut, din + 1, [&](int k, int p) { return p < din ? sG[k][0] * sA[k][p] : sG[k][0]; });
    }
    S da[kResMaxWidth];
#pragma unroll
    for (int i = 0; i < kResMaxWidth; ++i) da[i] = i < din ? dt * RM<S>::w(r, offOut + i) : S(0);
    // hidden layers, top down
    for (int l = H - 1; l >= (fin ? 0 : pass); --l) {
      S ain[kResMaxWidth];
      UdeLayer<S> L;
      int dl;
      ude_inputs(r, cc, h, qx, qy, ain);
      const int off = ude_forward_to(r, l, ain, L, dl);
      const int w = r.width[l];
      const int offLn = off + w * dl + w;
      S dxh[kResMaxWidth];
#pragma unroll
      for (int o = 0; o < kResMaxWidth; ++o) dxh[o] = o < w ? da[o] * RM<S>::w(r, offLn + o) : S(0);
      if (l == pass) {   // this pass's sums
        if (live) {
          S t1 = S(0), t2 = S(0);
#pragma unroll
          for (int o = 0; o < kResMaxWidth; ++o) {
            t1 += dxh[o];
            t2 += dxh[o] * L.xh[o];
          }
          s1 += (double)t1;
          s2 += (double)t2;
        }
        break;
      }
      S m1, m2;
      if (r.overBatch) {
        const double M = (double)n * (double)w;
        m1 = S(ad.udeS[2 * l] / M);
        m2 = S(ad.udeS[2 * l + 1] / M);
      } else {
        S t1 = S(0), t2 = S(0);
#pragma unroll
        for (int o = 0; o < kResMaxWidth; ++o) {
          t1 += dxh[o];
          t2 += dxh[o] * L.xh[o];
        }
        m1 = t1 / S(w);
        m2 = t2 / S(w);
      }
      S dp[kResMaxWidth];
#pragma unroll
      for (int o = 0; o < kResMaxWidth; ++o)
        dp[o] = (o < w && live) ? (dxh[o] - m1 - L.xh[o] * m2) / L.den * activation_grad(r.act[l], L.p[o], L.z[o])
                                : S(0);
      if (fin) {
#pragma unroll
        for (int i = 0; i < kResMaxWidth; ++i) {
          sA[lane][i] = ain[i];
          sG[lane][i] = dp[i];
          sX[lane][i] = L.xh[i];
          sD[lane][i] = da[i];
        }
        const int nw = w * dl;
        reduce(off, nw + 3 * w, [&](int k, int p) {
          if (p < nw) return sG[k][p % w] * sA[k][p / w];
          if (p < nw + w) return sG[k][p - nw];
          if (p < nw + 2 * w) return sD[k][p - nw - w] * sX[k][p - nw - w];
          return sD[k][p - nw - 2 * w];
        });
      }
#pragma unroll
      for (int i = 0; i < kResMaxWidth; ++i) {
        S s = S(0);
        if (i < dl) {
#pragma unroll
          for (int o = 0; o < kResMaxWidth; ++o)
            if (o < w) s += RM<S>::w(r, off + o + i * w) * dp[o];
        }
        da[i] = s;
      }
    }
    if (fin && live && !cell_dry(m, Q, c)) {   // inputs -> state (the clamp zeroes a dry cell's derivative)
      S gh = da[0] * S(2.0) / (S(r.hi[0]) - S(r.lo[0]));
      S gqx = S(0), gqy = S(0);
      if (r.kind == kResUdeManningHUmagKs) {   // Umag = |q| / h
        const S u = qx / h, v = qy / h;
        const S um = RM<S>::sqrt(u * u + v * v);
        if (um > S(0)) {
          const S gu = da[1] * S(2.0) / (S(r.hi[1]) - S(r.lo[1]));
          gh += gu * (-um / h);
          gqx = gu * u / (um * h);
          gqy = gu * v / (um * h);
        }
      } else if (r.kind == kResUdeFlowResistance) {   // |q| smoothed
        const S mag = smooth_sqrt(qx * qx + qy * qy);
        const S gq = da[1] * S(2.0) / (S(r.hi[0] * r.hi[1]) - S(r.lo[0] * r.lo[1]));
        gqx = gq * qx / mag;
        gqy = gq * qy / mag;
      }
      out[c] += gh;
      out[n + c] += gqx;
      out[2 * n + c] += gqy;
    }
  }
  // per-block sums, then the last block adds them in block order
  __shared__ int isLast;
  if (fin) {
    __syncwarp();
    for (int p = lane; p < P; p += 32) ad.udePart[(size_t)blockIdx.x * P + p] = sAcc[p];
  } else {
    s1 = warp_sum_d(s1);
    s2 = warp_sum_d(s2);
    if (lane == 0) {
      ad.udePart[2 * blockIdx.x] = s1;
      ad.udePart[2 * blockIdx.x + 1] = s2;
    }
  }
  __threadfence();
  __syncwarp();
  if (lane == 0) isLast = (atomicAdd(ad.udeTicket, 1u) == gridDim.x - 1);
  __syncwarp();
  if (!isLast) return;
  __threadfence();
  if (fin) {
    for (int p = lane; p < P; p += 32) {
      double t = 0.0;
      for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(&ad.udePart[(size_t)b * P + p]);
      ad.gTheta[p] += t;
    }
  } else {
    double t1 = 0.0, t2 = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) {
      t1 += __ldcg(&ad.udePart[2 * b]);
      t2 += __ldcg(&ad.udePart[2 * b + 1]);
    }
    t1 = warp_sum_d(t1);
    t2 = warp_sum_d(t2);
    if (lane == 0) {
      ad.udeS[2 * pass] = t1;
      ad.udeS[2 * pass + 1] = t2;
    }
  }
  if (lane == 0) *ad.udeTicket = 0u;
}

template <class S, class State, class Out>
int launch_ude_vjp(const DevMesh& m, const AdjDev& a, State Q, Out* out, cudaStream_t st) {
  if (!a.udeChain || m.n == 0) return 0;
  const int64_t rounds = (m.n + 31) / 32;
  const int grid = (int)(rounds < kUdeGrid ? rounds : kUdeGrid);
  int launches = 0;
  if (m.res.overBatch)
    for (int l = m.res.nHidden - 1; l >= 0; --l) {
      k_ude_vjp<S, State, Out><<<grid, 32, 0, st>>>(m, a, Q, out, l);
      ++launches;
    }
  k_ude_vjp<S, State, Out><<<grid, 32, 0, st>>>(m, a, Q, out, -1);
  return launches + 1;
}

}  // namespace

}  // namespace hg
