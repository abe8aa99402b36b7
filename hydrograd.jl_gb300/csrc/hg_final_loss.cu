// Final-state inversion loss of swe_2D_inversion.jl:383-431 (the WSE and
// velocity misfits of the last saved state) as a seed of the discrete adjoint:
// its value and its gradient w.r.t. the final state.  FP64 arithmetic on both
// paths (one pass over the cells per call).
#include <cmath>

#include "hg_adjoint_state.hpp"
#include "hg_reduce.cuh"
#include "hg_state.hpp"

namespace hg {

using namespace devred;

namespace {

constexpr int kBlock = 256;
constexpr double kSqrtEps = 1.4901161193847656e-08;   // sqrt(eps(Float64))

__device__ __forceinline__ void final_state(const DevMesh& m, const double* __restrict__ Q, int c, double& xi,
                                            double& qx, double& qy) {
  xi = Q[c];
  qx = Q[m.n + c];
  qy = Q[2 * m.n + c];
}
__device__ __forceinline__ void final_state(const DevMesh& m, StateF32 Q, int c, double& xi, double& qx, double& qy) {
  const float4 x = Q.x[c];
  const float2 q = Q.q[c];
  xi = (double)x.x + (double)x.y;
  qx = (double)x.z + (double)q.x;
  qy = (double)x.w + (double)q.y;
}

template <class State, class Mu>
__global__ void __launch_bounds__(kBlock) k_final_loss(DevMesh m, FinalLossDev f, State Q, Mu* mu) {
  double sw = 0.0, suv = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.n; c += gridDim.x * blockDim.x) {
    double xi, qx, qy;
    final_state(m, Q, c, xi, qx, qy);
    const double h = xi + m.hst[c];   // h_pred = xi_pred + hstill (no clamp)
    double gxi = 0.0, gqx = 0.0, gqy = 0.0;
    if (f.wse) {
      const double r = ((h + f.zbw[c]) - f.wse[c]) / f.wseDen;
      sw += r * r;
      const double d = 2.0 * r / f.wseDen * f.invN;
      gxi += d;
      f.dWse[c] = d;
    }
    if (f.u) {
      const double e = h + kSqrtEps;
      const double ru = (qx / e - f.u[c]) / f.velScale, rv = (qy / e - f.v[c]) / f.velScale;
      suv += ru * ru + rv * rv;
      const double du = 2.0 * ru / f.velScale * f.invN, dv = 2.0 * rv / f.velScale * f.invN;
      gqx += du / e;
      gqy += dv / e;
      gxi -= (du * qx + dv * qy) / (e * e);
    }
    if (f.lam) {
      gxi += f.lam[c];
      gqx += f.lam[m.n + c];
      gqy += f.lam[2 * m.n + c];
    }
    if (!f.mask || h > m.hsm) {   // a cell the last stage clamped does not depend on its inputs
      mu[c] += (Mu)gxi;
      mu[m.n + c] += (Mu)gqx;
      mu[2 * m.n + c] += (Mu)gqy;
    }
  }
  const double bw = block_sum(sw);
  const double buv = block_sum(suv);
  __shared__ int isLast;
  if (threadIdx.x == 0) {
    f.partials[2 * blockIdx.x] = bw;
    f.partials[2 * blockIdx.x + 1] = buv;
    __threadfence();
    isLast = (atomicAdd(f.ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!isLast) return;
  __threadfence();
  double tw = 0.0, tuv = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    tw += __ldcg(&f.partials[2 * k]);
    tuv += __ldcg(&f.partials[2 * k + 1]);
  }
  tw = block_sum(tw);
  tuv = block_sum(tuv);
  if (threadIdx.x == 0) {
    f.parts[0] = tw * f.invN;
    f.parts[1] = tuv * f.invN;
    *f.ticket = 0u;
  }
}

int grid_for(int n) {
  const int b = (n + kBlock - 1) / kBlock;
  return b < kFinalLossBlocks ? (b > 0 ? b : 1) : kFinalLossBlocks;
}

}  // namespace

void launch_final_loss_f64(const DevMesh& m, const FinalLossDev& f, const double* Q, double* mu, cudaStream_t st) {
  k_final_loss<const double*, double><<<grid_for(m.n), kBlock, 0, st>>>(m, f, Q, mu);
}

void launch_final_loss_f32(const DevMesh& m, const FinalLossDev& f, StateF32 Q, float* mu, cudaStream_t st) {
  k_final_loss<StateF32, float><<<grid_for(m.n), kBlock, 0, st>>>(m, f, Q, mu);
}

}  // namespace hg
