// Host driver of the Tsit5 integrator (hg_integrate_tsit5): adaptive steps of
// the Tsitouras 5(4) pair on the device RHS, with the step-size control of
// Hairer, Norsett & Wanner, "Solving ODEs I", II.4 (embedded error estimate in
// a weighted RMS norm, PI controller, Hairer's initial step).
//
// The state lives on the device in the device cell order: one FP64 vector
// U = [xi | qx | qy] in an FP64 context, hi + lo records in an
// FP32-compensated one (VecsF64 / VecsF32 below); each stage's RHS is the
// context's RHS kernel.
// As in the reference's ODE solve, the RHS clamps depths internally and the
// integrator adds no clamp of its own.  One 8-byte read-back per step (the
// error norm) drives the controller.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hg_ctx.hpp"
#include "hg_state.hpp"
#include "hg_tsit5.hpp"
#include "hydrograd_gb.h"

namespace hg {

const Tsit5Tableau& tsit5_tableau() {
  static const Tsit5Tableau t = [] {
    Tsit5Tableau r{};
    const double c[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
    const double a[7][7] = {
        {0, 0, 0, 0, 0, 0, 0},
        {0.161, 0, 0, 0, 0, 0, 0},
        {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0, 0},
        {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0, 0},
        {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0, 0},
        {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0, 0},
        {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774,
         0}};
    const double bt[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                          -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152};
    for (int i = 0; i < 7; ++i) {
      r.c[i] = c[i];
      r.b[i] = a[6][i];
      r.btilde[i] = bt[i];
      for (int j = 0; j < 7; ++j) r.a[i][j] = a[i][j];
    }
    return r;
  }();
  return t;
}

namespace {

int fail(hg_ctx* c, int code, const std::string& m) {
  c->err = m;
  return code;
}

#define TS_CUDA(c, call)                                                                         \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail((c), HG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device buffers of one run (freed on return).
struct Tsit5Buffers {
  std::vector<void*> ptrs;
  ~Tsit5Buffers() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e == cudaSuccess) {
      ptrs.push_back(q);
      *p = static_cast<T*>(q);
    }
    return e;
  }
};

// The integrator's vectors and kernels by precision.  FP64 contexts: plain
// [3n] FP64 vectors, the FP64 RHS, combinations and norm in FP64 (the
// oracle's arithmetic).  FP32-compensated contexts: stage states as hi + lo
// records, RHS vectors in FP32 (the FP32 stage kernel's own precision), the
// weighted sums in FP32 added to the states with compensated sums, the norm's
// terms in FP32 -- GB300 issues FP64 at a small fraction of the FP32 rate, and
// the FP64 combinations were most of an FP32-compensated step.
struct VecsF64 {
  using State = double*;
  using Deriv = double*;
  hg_ctx* c;
  double abstol, reltol;
  double *partials, *norm2;
  unsigned int* ticket;
  int64_t len() const { return (int64_t)3 * c->n; }
  cudaError_t alloc(Tsit5Buffers& B, State& v) { return B.alloc(&v, len()); }
  cudaError_t allocD(Tsit5Buffers& B, Deriv& v) { return B.alloc(&v, len()); }
  void load(State U) { launch_gather_state_f64(c->n, c->d_perm, c->Quser, U, c->stream); }
  void unload(State U) { launch_scatter_state_f64(c->n, c->d_perm, U, c->Quser, c->stream); }
  void rhs(State X, Deriv out) {
    launch_inlet_total_f64(c->dm, c->ds, X, c->stream);
    launch_stage_f64(c->dm, c->ds, kModeRhs, X, nullptr, out, false, c->stream);
  }
  static Tsit5Terms terms(const Deriv* K, const double* w, int nk) {
    Tsit5Terms t{};
    for (int j = 0; j < nk; ++j) {
      t.K[j] = K[j];
      t.w[j] = w[j];
    }
    t.nk = nk;
    return t;
  }
  void combine(State U, const Deriv* K, const double* w, int nk, double h, State Y) {
    launch_tsit5_combine(len(), U, terms(K, w, nk), h, Y, c->stream);
  }
  void error(State Ua, State Ub, const Deriv* K, const double* w, int nk, double h) {
    launch_tsit5_error(len(), Ua, Ub, terms(K, w, nk), h, abstol, reltol, partials, ticket, norm2, c->stream);
  }
  void state_norm(State U) {   // the state itself as the vector
    const double one = 1.0;
    launch_tsit5_error(len(), U, U, terms(&U, &one, 1), 1.0, abstol, reltol, partials, ticket, norm2, c->stream);
  }
};

struct VecsF32 {
  using State = StateF32;
  using Deriv = float*;
  hg_ctx* c;
  double abstol, reltol;
  double *partials, *norm2;
  unsigned int* ticket;
  int64_t len() const { return (int64_t)3 * c->n; }
  cudaError_t alloc(Tsit5Buffers& B, State& v) {
    cudaError_t e = B.alloc(&v.x, (size_t)c->n);
    return e == cudaSuccess ? B.alloc(&v.q, (size_t)c->n) : e;
  }
  cudaError_t allocD(Tsit5Buffers& B, Deriv& v) { return B.alloc(&v, len()); }
  void load(State U) { launch_gather_state_f32(c->n, c->d_perm, c->Quser, U, c->stream); }
  void unload(State U) { launch_scatter_state_f32(c->n, c->d_perm, U, c->Quser, c->stream); }
  void rhs(State X, Deriv out) {
    launch_inlet_total_f32(c->dm, c->ds, X, c->stream);
    launch_stage_f32(c->dm, c->ds, kModeRhsF32, X, StateF32{}, StateF32{}, reinterpret_cast<double*>(out), false,
                     c->stream);
  }
  static Tsit5TermsF terms(const Deriv* K, const double* w, int nk, double h) {
    Tsit5TermsF t{};
    for (int j = 0; j < nk; ++j) {
      t.K[j] = K[j];
      t.w[j] = (float)(w[j] * h);
    }
    t.nk = nk;
    return t;
  }
  void combine(State U, const Deriv* K, const double* w, int nk, double h, State Y) {
    launch_tsit5_combine_f32(c->n, U, terms(K, w, nk, h), Y, c->stream);
  }
  void error(State Ua, State Ub, const Deriv* K, const double* w, int nk, double h) {
    launch_tsit5_error_f32(c->n, Ua, Ub, terms(K, w, nk, h), (float)abstol, (float)reltol, partials, ticket, norm2,
                           c->stream);
  }
  void state_norm(State U) {
    launch_tsit5_error_f32(c->n, U, U, Tsit5TermsF{}, (float)abstol, (float)reltol, partials, ticket, norm2,
                           c->stream);
  }
};

template <class V>
int run_tsit5(hg_ctx* ctx, V& vec, double* Q, double t0, double t1, double dt0, int32_t adaptive, int32_t max_steps,
              int32_t n_save, const double* t_save, double* saves, int32_t* stats);

}  // namespace
}  // namespace hg

using namespace hg;

int hg_tsit5_tableau(double* c7, double* a49, double* b7, double* btilde7) {
  const Tsit5Tableau& t = tsit5_tableau();
  for (int i = 0; i < kTsit5Stages; ++i) {
    if (c7) c7[i] = t.c[i];
    if (b7) b7[i] = t.b[i];
    if (btilde7) btilde7[i] = t.btilde[i];
    for (int j = 0; j < kTsit5Stages; ++j)
      if (a49) a49[i * kTsit5Stages + j] = t.a[i][j];
  }
  return HG_OK;
}

int hg_integrate_tsit5(hg_ctx* ctx, double* Q, double t0, double t1, double abstol, double reltol, double dt0,
                       int32_t adaptive, int32_t max_steps, int32_t n_save, const double* t_save, double* saves,
                       int32_t* stats) {
  if (!ctx) return HG_ERR_ARG;
  if (!Q || !(t1 > t0) || !(abstol > 0) || !(reltol >= 0) || n_save < 0 || (n_save > 0 && (!t_save || !saves)))
    return fail(ctx, HG_ERR_ARG, "hg_integrate_tsit5: bad argument");
  if (!adaptive && !(dt0 > 0)) return fail(ctx, HG_ERR_ARG, "hg_integrate_tsit5: fixed steps need dt0 > 0");
  for (int i = 0; i < n_save; ++i)
    if (!(t_save[i] > t0 && t_save[i] <= t1) || (i > 0 && !(t_save[i] > t_save[i - 1])))
      return fail(ctx, HG_ERR_ARG, "hg_integrate_tsit5: save times must ascend within (t0, t1]");
  if (max_steps <= 0) max_steps = 10000000;
  cudaSetDevice(ctx->device);
  if (ctx->precision == HG_FP64) {
    VecsF64 v{ctx, abstol, reltol, nullptr, nullptr, nullptr};
    return run_tsit5(ctx, v, Q, t0, t1, dt0, adaptive, max_steps, n_save, t_save, saves, stats);
  }
  VecsF32 v{ctx, abstol, reltol, nullptr, nullptr, nullptr};
  return run_tsit5(ctx, v, Q, t0, t1, dt0, adaptive, max_steps, n_save, t_save, saves, stats);
}

namespace hg {
namespace {

template <class V>
int run_tsit5(hg_ctx* ctx, V& vec, double* Q, double t0, double t1, double dt0, int32_t adaptive, int32_t max_steps,
              int32_t n_save, const double* t_save, double* saves, int32_t* stats) {
  using State = typename V::State;
  using Deriv = typename V::Deriv;
  const Tsit5Tableau& tb = tsit5_tableau();
  const int n = ctx->n;
  const int64_t len = (int64_t)3 * n;
  cudaStream_t st = ctx->stream;
  Tsit5Buffers B;
  State U{}, Unew{}, Y{};
  Deriv K[kTsit5Stages];
  TS_CUDA(ctx, vec.alloc(B, U));
  TS_CUDA(ctx, vec.alloc(B, Unew));
  TS_CUDA(ctx, vec.alloc(B, Y));
  for (auto& k : K) TS_CUDA(ctx, vec.allocD(B, k));
  TS_CUDA(ctx, B.alloc(&vec.partials, kTsit5ErrorBlocks));
  TS_CUDA(ctx, B.alloc(&vec.norm2, 1));
  TS_CUDA(ctx, B.alloc(&vec.ticket, 1));
  TS_CUDA(ctx, cudaMemsetAsync(vec.ticket, 0, sizeof(unsigned int), st));
  TS_CUDA(ctx, cudaMemsetAsync(ctx->ds.flags, 0, sizeof(int32_t), st));
  // State in: caller order -> device order.
  TS_CUDA(ctx, cudaMemcpyAsync(ctx->Quser, Q, len * sizeof(double), cudaMemcpyHostToDevice, st));
  vec.load(U);
  ctx->launches += 1;
  auto rhs = [&](State X, Deriv out, double tx) {
    ctx->launches += launch_hydrograph(ctx->dm, ctx->ds, kHydroAt, tx, st);   // inlet discharges at tx
    vec.rhs(X, out);
    ctx->launches += 1 + (ctx->dm.nInlet > 0 ? 1 : 0) + resistance_launches(ctx->dm);
  };
  // Weighted RMS norm (scale abstol + reltol max(|Ua|, |Ub|)) of the vector
  // the last error launch formed.
  auto read_norm = [&](double& out) -> int {
    ctx->launches += 1;
    double v = 0.0;
    TS_CUDA(ctx, cudaMemcpyAsync(&v, vec.norm2, sizeof(double), cudaMemcpyDeviceToHost, st));
    TS_CUDA(ctx, cudaStreamSynchronize(st));
    out = std::sqrt(v / (double)len);
    return HG_OK;
  };
  const double unit = 1.0;
  rhs(U, K[0], t0);
  double dt = dt0;
  if (adaptive && !(dt > 0)) {   // Hairer, Norsett & Wanner II.4: starting step size
    double d0, d1, d2;
    vec.state_norm(U);
    int rc = read_norm(d0);
    if (!rc) {
      vec.error(U, U, K, &unit, 1, 1.0);
      rc = read_norm(d1);
    }
    if (rc) return rc;
    const double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    vec.combine(U, K, &unit, 1, h0, Y);
    rhs(Y, K[1], t0 + h0);
    const Deriv dk[2] = {K[1], K[0]};
    const double wk[2] = {1.0 / h0, -1.0 / h0};
    vec.error(U, U, dk, wk, 2, 1.0);
    rc = read_norm(d2);
    if (rc) return rc;
    const double m = std::max(d1, d2);
    const double h1 = m <= 1e-15 ? std::max(1e-6, h0 * 1e-3) : std::pow(0.01 / m, 1.0 / 5.0);
    dt = std::min(100.0 * h0, h1);
  }
  if (adaptive) dt = std::min(dt, t1 - t0);
  // PI controller (Hairer & Wanner II.4): gains for a method of order 5.
  const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, gamma = 0.9, qmin = 0.2, qmax = 10.0;
  double errOld = 1e-4;
  double t = t0;
  int accepted = 0, rejected = 0, saved = 0;
  ctx->tsit5Steps.clear();
  int evals = (adaptive && !(dt0 > 0)) ? 2 : 1;   // RHS evaluations so far: K1, and the starting-step probe
  while (t1 - t > 1e-14 * std::max(1.0, std::fabs(t1))) {
    if (accepted + rejected >= max_steps) return fail(ctx, HG_ERR_ARG, "hg_integrate_tsit5: max_steps reached");
    const double target = saved < n_save ? t_save[saved] : t1;
    double h = dt;
    bool hit = false;
    if (t + h >= target - 1e-14 * std::max(1.0, std::fabs(target))) {
      h = target - t;
      hit = true;
    }
    for (int i = 1; i < kTsit5Stages; ++i) {   // stages 2..7; stage 7's state is the new state
      State dst = (i == kTsit5Stages - 1) ? Unew : Y;
      vec.combine(U, K, tb.a[i], i, h, dst);
      rhs(dst, K[i], t + tb.c[i] * h);
      ctx->launches += 1;
    }
    evals += kTsit5Stages - 1;
    double eest = 0.0;
    if (adaptive) {
      vec.error(U, Unew, K, tb.btilde, kTsit5Stages, h);
      int rc = read_norm(eest);
      if (rc) return rc;
    }
    if (eest <= 1.0) {
      ctx->tsit5Steps.push_back(h);
      t = hit ? target : t + h;
      std::swap(U, Unew);
      std::swap(K[0], K[kTsit5Stages - 1]);   // first same as last
      ++accepted;
      if (adaptive) {
        const double fac = std::min(qmax, std::max(qmin, gamma * std::pow(std::max(eest, 1e-12), -beta1) *
                                                              std::pow(errOld, beta2)));
        errOld = std::max(eest, 1e-4);
        dt = h * fac;
      }
      if (hit && saved < n_save) {
        vec.unload(U);
        ctx->launches += 1;
        TS_CUDA(ctx, cudaMemcpyAsync(saves + (size_t)saved * len, ctx->Quser, len * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
        ++saved;
      }
    } else {
      ++rejected;
      const double fac = std::isfinite(eest) ? std::max(qmin, gamma * std::pow(eest, -beta1)) : qmin;
      dt = h * fac;
      if (dt < 1e-14 * std::max(1.0, std::fabs(t)))
        return fail(ctx, HG_ERR_STATE, "hg_integrate_tsit5: step size underflow");
    }
  }
  vec.unload(U);
  ctx->launches += 1;
  TS_CUDA(ctx, cudaMemcpyAsync(Q, ctx->Quser, len * sizeof(double), cudaMemcpyDeviceToHost, st));
  int32_t flags = 0;
  TS_CUDA(ctx, cudaMemcpyAsync(&flags, ctx->ds.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  TS_CUDA(ctx, cudaStreamSynchronize(st));
  if (stats) {
    stats[0] = accepted;
    stats[1] = rejected;
    stats[2] = evals;
  }
  if (flags & 2) return fail(ctx, HG_ERR_INLET, "inlet-Q total conveyance is not positive (all inlet cells dry?)");
  if (flags & 1) return fail(ctx, HG_ERR_STATE, "non-finite value in the state");
  return HG_OK;
}

}  // namespace
}  // namespace hg
