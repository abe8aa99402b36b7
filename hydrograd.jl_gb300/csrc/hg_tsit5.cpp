// Host driver of the Tsit5 integrator (hg_integrate_tsit5): adaptive steps of
// the Tsitouras 5(4) pair on the device RHS, with the step-size control of
// Hairer, Norsett & Wanner, "Solving ODEs I", II.4 (embedded error estimate in
// a weighted RMS norm, PI controller, Hairer's initial step).
//
// The state lives on the device as one FP64 vector U = [xi | qx | qy] in the
// device cell order; each stage's RHS is the context's RHS kernel (FP64, or
// the FP32-compensated kernel on the stage state split into hi + lo pairs).
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
  const Tsit5Tableau& tb = tsit5_tableau();
  const int n = ctx->n;
  const int64_t len = (int64_t)3 * n;
  cudaStream_t st = ctx->stream;
  Tsit5Buffers B;
  double *U, *Unew, *Y, *K[kTsit5Stages], *partials, *norm2;
  unsigned int* ticket;
  TS_CUDA(ctx, B.alloc(&U, len));
  TS_CUDA(ctx, B.alloc(&Unew, len));
  TS_CUDA(ctx, B.alloc(&Y, len));
  for (auto& k : K) TS_CUDA(ctx, B.alloc(&k, len));
  TS_CUDA(ctx, B.alloc(&partials, kTsit5ErrorBlocks));
  TS_CUDA(ctx, B.alloc(&norm2, 1));
  TS_CUDA(ctx, B.alloc(&ticket, 1));
  TS_CUDA(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st));
  TS_CUDA(ctx, cudaMemsetAsync(ctx->ds.flags, 0, sizeof(int32_t), st));
  // State in: caller order -> device order.
  TS_CUDA(ctx, cudaMemcpyAsync(ctx->Quser, Q, len * sizeof(double), cudaMemcpyHostToDevice, st));
  launch_gather_state_f64(n, ctx->d_perm, ctx->Quser, U, st);
  ctx->launches += 1;
  const StateF32 xs{ctx->XB, ctx->XQB};
  auto rhs = [&](const double* X, double* out, double tx) {
    ctx->launches += launch_hydrograph(ctx->dm, ctx->ds, kHydroAt, tx, st);   // inlet discharges at tx
    if (ctx->precision == HG_FP64) {
      launch_inlet_total_f64(ctx->dm, ctx->ds, X, st);
      launch_stage_f64(ctx->dm, ctx->ds, kModeRhs, X, nullptr, out, false, st);
    } else {
      launch_f64_to_f32(n, X, xs, st);
      launch_inlet_total_f32(ctx->dm, ctx->ds, xs, st);
      launch_stage_f32(ctx->dm, ctx->ds, kModeRhs, xs, StateF32{}, StateF32{}, out, false, st);
      ctx->launches += 1;
    }
    ctx->launches += 1 + (ctx->dm.nInlet > 0 ? 1 : 0) + resistance_launches(ctx->dm);
  };
  // Weighted RMS norm of sum_j w_j V_j (scale abstol + reltol max(|Ua|, |Ub|)).
  auto wnorm = [&](const double* Ua, const double* Ub, Tsit5Terms terms, double h, double& out) -> int {
    launch_tsit5_error(len, Ua, Ub, terms, h, abstol, reltol, partials, ticket, norm2, st);
    ctx->launches += 1;
    double v = 0.0;
    TS_CUDA(ctx, cudaMemcpyAsync(&v, norm2, sizeof(double), cudaMemcpyDeviceToHost, st));
    TS_CUDA(ctx, cudaStreamSynchronize(st));
    out = std::sqrt(v / (double)len);
    return HG_OK;
  };
  auto one = [](const double* v, double w) {
    Tsit5Terms t{};
    t.K[0] = v;
    t.w[0] = w;
    t.nk = 1;
    return t;
  };
  rhs(U, K[0], t0);
  double dt = dt0;
  if (adaptive && !(dt > 0)) {   // Hairer, Norsett & Wanner II.4: starting step size
    double d0, d1, d2;
    int rc = wnorm(U, U, one(U, 1.0), 1.0, d0);
    if (!rc) rc = wnorm(U, U, one(K[0], 1.0), 1.0, d1);
    if (rc) return rc;
    const double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    launch_tsit5_combine(len, U, one(K[0], 1.0), h0, Y, st);
    rhs(Y, K[1], t0 + h0);
    Tsit5Terms dk{};
    dk.K[0] = K[1];
    dk.K[1] = K[0];
    dk.w[0] = 1.0 / h0;
    dk.w[1] = -1.0 / h0;
    dk.nk = 2;
    rc = wnorm(U, U, dk, 1.0, d2);
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
      Tsit5Terms terms{};
      for (int j = 0; j < i; ++j) {
        terms.K[j] = K[j];
        terms.w[j] = tb.a[i][j];
      }
      terms.nk = i;
      double* dst = (i == kTsit5Stages - 1) ? Unew : Y;
      launch_tsit5_combine(len, U, terms, h, dst, st);
      rhs(dst, K[i], t + tb.c[i] * h);
      ctx->launches += 1;
    }
    evals += kTsit5Stages - 1;
    double eest = 0.0;
    if (adaptive) {
      Tsit5Terms et{};
      for (int j = 0; j < kTsit5Stages; ++j) {
        et.K[j] = K[j];
        et.w[j] = tb.btilde[j];
      }
      et.nk = kTsit5Stages;
      int rc = wnorm(U, Unew, et, h, eest);
      if (rc) return rc;
    }
    if (eest <= 1.0) {
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
        launch_scatter_state_f64(n, ctx->d_perm, U, ctx->Quser, st);
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
  launch_scatter_state_f64(n, ctx->d_perm, U, ctx->Quser, st);
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
