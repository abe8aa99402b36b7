// FP32-compensated stage kernels, step bookkeeping and renumbering kernels.
//
// Forward kernels: one fused pass per explicit stage.
//
// Each thread owns one cell (device order) and gathers its faces in the
// reference's local order (compute_inviscid_fluxes,
// src/fvm/discretization/semi_discretize_swe_2D.jl:286-419): clamp, ghost
// state, Roe flux, -sum F L / A, Manning friction + bed-slope source, then the
// stage update and the depth-positivity clamp.  Gather form: no atomics, and
// the per-cell summation order is the reference's, so the result is
// deterministic and independent of the launch shape.
#include <cfloat>
#include <cmath>

#include "hg_device.cuh"
#include "hg_reduce.cuh"
#include "hg_state.hpp"

namespace hg {

using namespace hgd;

namespace {

constexpr int kBlock = 256;

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

using namespace devred;

// ---------------------------------------------------------------------------
// FP32-compensated path
// ---------------------------------------------------------------------------
// State components are hi + lo float pairs; hstill is an exact hi + lo pair.
// Depth h = xi + hstill: the dry decision h <= h_small is taken exactly as the
// FP64 reference takes it -- from an FP32 estimate when that estimate is
// farther from h_small than its error bound, else from an FP64 sum -- with a
// tolerance of a few units of the pair representation (2^-46 relative), the
// granularity at which a clamped cell's xi = h_small - hstill is stored.
struct DepthF32 {
  float h;        // clamped depth
  float excess;   // (h_clamped - hstill) - xi: 0 when wet, the clamp shift when dry
  bool dry;
};

__device__ __forceinline__ DepthF32 depth_f32(float xh, float xl, float hh, float hl, float hsmf, double hsm) {
  DepthF32 d;
  const float est = (xh + hh) + (xl + hl);
  const float mag = fabsf(xh) + fabsf(hh);
  const float bound = 4.0e-7f * mag + 1.0e-30f;
  if (fabsf(est - hsmf) > bound + 1.0e-10f) {
    d.dry = est <= hsmf;
    d.h = est;
  } else {
    const double hd = ((double)xh + (double)xl) + ((double)hh + (double)hl);
    const double tol = 1.4210854715202004e-14 * (double)mag;   // 2^-46 * magnitude
    d.dry = hd <= hsm + tol;
    d.h = (float)hd;
  }
  d.excess = d.dry ? (hsmf - est) : 0.0f;
  if (d.dry) d.h = hsmf;
  return d;
}

struct SideF32 {
  Side<float> s;
  float xlo;      // lo part of xi
  float excess;
};

__device__ __forceinline__ SideF32 load_f32(const DevMesh& m, const float* __restrict__ Xh, const float* __restrict__ Xl,
                                            int j, float hsmf) {
  SideF32 r;
  const float xh = Xh[j], xl = Xl[j];
  const float hh = m.hsthi[j], hl = m.hstlo[j];
  const DepthF32 d = depth_f32(xh, xl, hh, hl, hsmf, m.hsm);
  r.s.xi = xh;
  r.xlo = xl;
  r.s.hst = hh;
  r.s.zb = m.zbf[j];
  r.s.dry = d.dry;
  r.s.h = d.h;
  r.s.hu = d.dry ? 0.0f : Xh[m.n + j];
  r.s.hv = d.dry ? 0.0f : Xh[2 * m.n + j];
  r.excess = d.excess;
  return r;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// (ah + al) + d, renormalised.
__device__ __forceinline__ void df_add(float ah, float al, float d, float& rh, float& rl) {
  float s, e;
  two_sum(ah, d, s, e);
  e += al;
  fast_two_sum(s, e, rh, rl);
}
// (ah + al) + (bh + bl), renormalised.
__device__ __forceinline__ void df_add2(float ah, float al, float bh, float bl, float& rh, float& rl) {
  float s, e;
  two_sum(ah, bh, s, e);
  e += al + bl;
  fast_two_sum(s, e, rh, rl);
}

__device__ __forceinline__ void face_sum_f32(const DevMesh& m, const float* __restrict__ Xh,
                                             const float* __restrict__ Xl, int c, const SideF32& L, float hsmf,
                                             float g, float& f0, float& f1, float& f2) {
  f0 = 0.0f; f1 = 0.0f; f2 = 0.0f;
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * m.n + c];
    if (nb == kNoFace) break;
    const float nx = m.snxf[(size_t)k * m.n + c], ny = m.snyf[(size_t)k * m.n + c];
    const float len = m.slenf[(size_t)k * m.n + c];
    Side<float> R;
    float dxi;
    if (nb >= 0) {
      const SideF32 r = load_f32(m, Xh, Xl, nb, hsmf);
      R = r.s;
      dxi = (r.s.xi - L.s.xi) + (r.xlo - L.xlo);
    } else {
      const int32_t bf = boundary_index(nb);
      const int32_t info = m.bfInfo[bf], type = info & 3, grp = info >> 2;
      R = ghost_state<float>(L.s, type, nx, ny, hsmf, type == kBcExitH ? (float)m.exitWse[grp] : 0.0f,
                             type == kBcInletQ ? (float)m.inletQ[grp] : 0.0f,
                             type == kBcInletQ ? (float)m.totalA[grp] : 1.0f, m.bfLp23f[bf], m.manf[c]);
      // xi_ghost - xi = (h_ghost - h) + ((h - hstill) - xi)
      dxi = (R.h - L.s.h) + L.excess;
    }
    float F[3];
    roe_flux<float>(L.s, R, dxi, g, nx, ny, hsmf, F);
    f0 = fmaf(F[0], len, f0);
    f1 = fmaf(F[1], len, f1);
    f2 = fmaf(F[2], len, f2);
  }
}

__device__ __forceinline__ float cfl_candidate_f32(const DevMesh& m, int c, float h, float qx, float qy, bool dry,
                                                   float g) {
  if (dry) { qx = 0.0f; qy = 0.0f; }
  const float u = qx / h, v = qy / h, a = sqrtf(g * h);
  float s = 0.0f;
  for (int k = 0; k < m.nslot; ++k) {
    const int32_t nb = m.nb[(size_t)k * m.n + c];
    if (nb == kNoFace) break;
    s += m.slenf[(size_t)k * m.n + c] * (fabsf(u * m.snxf[(size_t)k * m.n + c] + v * m.snyf[(size_t)k * m.n + c]) + a);
  }
  return m.areaf[c] / s;
}

__global__ void __launch_bounds__(kBlock) k_stage_f32(DevMesh m, DevScalars s, int mode, StateF32 Xin, StateF32 Xbase,
                                                      StateF32 Xout, double* Rout, int cfl) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = c < m.n;
  const float hsmf = (float)m.hsm, g = (float)m.g;
  float cand = INFINITY;
  if (active) {
    const SideF32 L = load_f32(m, Xin.hi, Xin.lo, c, hsmf);
    float f0, f1, f2;
    face_sum_f32(m, Xin.hi, Xin.lo, c, L, hsmf, g, f0, f1, f2);
    const float A = m.areaf[c];
    const float r0 = -f0 / A, r1 = -f1 / A, r2 = -f2 / A;
    const float fr = friction_coef(g, (float)m.kn2, hsmf, m.manf[c], L.s.h, L.s.hu, L.s.hv);
    const float sx = L.s.dry ? 0.0f : (g * L.s.xi * m.s0xf[c] - fr * L.s.hu);
    const float sy = L.s.dry ? 0.0f : (g * L.s.xi * m.s0yf[c] - fr * L.s.hv);
    const float d0 = r0, d1 = r1 + sx, d2 = r2 + sy;
    if (mode == kModeRhs) {
      Rout[c] = d0; Rout[m.n + c] = d1; Rout[2 * m.n + c] = d2;
    } else {
      const float dt = *s.dtf;
      const float inc[3] = {dt * d0, dt * d1, dt * d2};
      float xh[3], xl[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const size_t i = (size_t)b * m.n + c;
        if (mode == kModeStage2) {
          float sh, sl;
          df_add2(Xbase.hi[i], Xbase.lo[i], Xin.hi[i], Xin.lo[i], sh, sl);
          df_add(sh, sl, inc[b], xh[b], xl[b]);
          xh[b] *= 0.5f;
          xl[b] *= 0.5f;
        } else {
          df_add(Xin.hi[i], Xin.lo[i], inc[b], xh[b], xl[b]);
        }
      }
      const float hh = m.hsthi[c], hl = m.hstlo[c];
      DepthF32 dn = depth_f32(xh[0], xl[0], hh, hl, hsmf, m.hsm);
      bool clamp;
      if (mode == kModeEulerRef) {
        clamp = (double)xh[0] + (double)xl[0] < m.hsm;
      } else {
        clamp = dn.dry;   // h <= h_small (within the pair granularity): h = h_small, q = 0
      }
      if (clamp) {
        const double x0 = (mode == kModeEulerRef) ? m.hsm : dry_xi(m.hsm, (double)hh + (double)hl);
        xh[0] = (float)x0;
        xl[0] = (float)(x0 - (double)xh[0]);
        xh[1] = xl[1] = xh[2] = xl[2] = 0.0f;
        dn.dry = true;
        dn.h = hsmf;
      }
      if (!(isfinite(xh[0]) && isfinite(xh[1]) && isfinite(xh[2]))) atomicOr(s.flags, 1);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        Xout.hi[(size_t)b * m.n + c] = xh[b];
        Xout.lo[(size_t)b * m.n + c] = xl[b];
      }
      if (cfl) cand = cfl_candidate_f32(m, c, dn.h, xh[1], xh[2], dn.dry, g);
    }
  }
  if (cfl) block_min_publish_f(cand, s.cflMinF);
}

__global__ void __launch_bounds__(kBlock) k_cfl_f32(DevMesh m, DevScalars s, StateF32 X) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  float cand = INFINITY;
  if (c < m.n) {
    const float hsmf = (float)m.hsm;
    const SideF32 L = load_f32(m, X.hi, X.lo, c, hsmf);
    cand = cfl_candidate_f32(m, c, L.s.h, X.hi[m.n + c], X.hi[2 * m.n + c], L.s.dry, (float)m.g);
  }
  block_min_publish_f(cand, s.cflMinF);
}

__global__ void __launch_bounds__(kBlock) k_inlet_total_f32(DevMesh m, DevScalars s, StateF32 X) {
  const int g = blockIdx.x;
  const int o0 = m.inletOff[g], o1 = m.inletOff[g + 1];
  const float hsmf = (float)m.hsm;
  double acc = 0.0;
  for (int i = o0 + threadIdx.x; i < o1; i += blockDim.x) {
    const int c = m.inletCell[i];
    const SideF32 L = load_f32(m, X.hi, X.lo, c, hsmf);
    acc += L.s.dry ? 0.0 : m.inletLp53[i] * (double)L.s.h / (double)m.manf[c];
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) {
    m.totalA[g] = t;
    if (!(t > 1e-10)) atomicOr(s.flags, 2);
  }
}

// ---------------------------------------------------------------------------
// Bookkeeping and renumbering
// ---------------------------------------------------------------------------
__global__ void k_step_begin(DevScalars s, int cflMode, double cfl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (cflMode) {
    const double m = fmin(__longlong_as_double((long long)*s.cflMin), (double)__uint_as_float(*s.cflMinF));
    *s.dt = cfl * m;
    *s.cflMin = (unsigned long long)__double_as_longlong(INFINITY);
    *s.cflMinF = __float_as_uint(INFINITY);
  }
  *s.dtf = (float)*s.dt;
  const int k = *s.stepIdx;
  if (k < s.dtCap) s.dtHist[k] = *s.dt;
  *s.stepIdx = k + 1;
  *s.tSum += *s.dt;
}

__global__ void k_reset_scalars(DevScalars s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  *s.cflMin = (unsigned long long)__double_as_longlong(INFINITY);
  *s.cflMinF = __float_as_uint(INFINITY);
  *s.stepIdx = 0;
  *s.tSum = 0.0;
  *s.flags = 0;
}

__global__ void k_gather_f64(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ user,
                             double* __restrict__ dev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  dev[i] = user[o];
  dev[n + i] = user[n + o];
  dev[2 * n + i] = user[2 * n + o];
}

__global__ void k_scatter_f64(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ dev,
                              double* __restrict__ user) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  user[o] = dev[i];
  user[n + o] = dev[n + i];
  user[2 * n + o] = dev[2 * n + i];
}

__global__ void k_gather_f32(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ user, StateF32 X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const double v = user[(size_t)b * n + o];
    const float h = (float)v;
    X.hi[(size_t)b * n + i] = h;
    X.lo[(size_t)b * n + i] = (float)(v - (double)h);
  }
}

__global__ void k_scatter_f32(int32_t n, const int32_t* __restrict__ perm, StateF32 X, double* __restrict__ user) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
#pragma unroll
  for (int b = 0; b < 3; ++b)
    user[(size_t)b * n + o] = (double)X.hi[(size_t)b * n + i] + (double)X.lo[(size_t)b * n + i];
}

__global__ void k_flush(uint4* buf, size_t n16) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4((unsigned)i, 1u, 2u, 3u);
}

}  // namespace
void launch_inlet_total_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st) {
  if (m.nInlet > 0) k_inlet_total_f32<<<m.nInlet, kBlock, 0, st>>>(m, s, X);
}
void launch_stage_f32(const DevMesh& m, const DevScalars& s, int mode, StateF32 Xin, StateF32 Xbase, StateF32 Xout,
                      double* Rout, bool cfl, cudaStream_t st) {
  k_stage_f32<<<blocks_for(m.n), kBlock, 0, st>>>(m, s, mode, Xin, Xbase, Xout, Rout, cfl ? 1 : 0);
}
void launch_cfl_f32(const DevMesh& m, const DevScalars& s, StateF32 X, cudaStream_t st) {
  k_cfl_f32<<<blocks_for(m.n), kBlock, 0, st>>>(m, s, X);
}
void launch_step_begin(const DevScalars& s, bool cflMode, double cfl, cudaStream_t st) {
  k_step_begin<<<1, 32, 0, st>>>(s, cflMode ? 1 : 0, cfl);
}
void launch_reset_scalars(const DevScalars& s, cudaStream_t st) { k_reset_scalars<<<1, 32, 0, st>>>(s); }
void launch_gather_state_f64(int32_t n, const int32_t* perm, const double* user, double* dev, cudaStream_t st) {
  k_gather_f64<<<blocks_for(n), kBlock, 0, st>>>(n, perm, user, dev);
}
void launch_scatter_state_f64(int32_t n, const int32_t* perm, const double* dev, double* user, cudaStream_t st) {
  k_scatter_f64<<<blocks_for(n), kBlock, 0, st>>>(n, perm, dev, user);
}
void launch_gather_state_f32(int32_t n, const int32_t* perm, const double* user, StateF32 dev, cudaStream_t st) {
  k_gather_f32<<<blocks_for(n), kBlock, 0, st>>>(n, perm, user, dev);
}
void launch_scatter_state_f32(int32_t n, const int32_t* perm, StateF32 dev, double* user, cudaStream_t st) {
  k_scatter_f32<<<blocks_for(n), kBlock, 0, st>>>(n, perm, dev, user);
}
void launch_flush(void* buf, size_t bytes, cudaStream_t st) {
  k_flush<<<152 * 8, 256, 0, st>>>(static_cast<uint4*>(buf), bytes / 16);
}

}  // namespace hg