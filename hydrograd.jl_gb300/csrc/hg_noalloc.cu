// hg_rhs_device_noalloc: the FP64 right-hand side for callers that cannot
// allocate device memory while they run.
//
// Some callers must not call cudaMalloc once their time loop has started: a
// Julia ODE integrator stepping inside CUDA.jl's memory pool, or a solver that
// records its step into a CUDA graph (stream capture forbids allocation and
// any call that may synchronise the device).  They create a context once, at
// set-up, keep their own state buffers, and then need an RHS evaluation that
// allocates nothing.  The RHS needs scratch memory for the inlet-Q conveyance
// totals (one per inlet boundary, bc_2D.jl:673-679) and an error-flag word; in
// the context these live in buffers that hg_create allocates.  Here they live
// in the file-scope array below instead, whose size is fixed at build time.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call rewrites the totals and clears the flag word before use.
// Calls that overlap on the GPU (different streams, no ordering between them)
// race on it.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "hg_ctx.hpp"
#include "hg_state.hpp"
#include "hydrograd_gb.h"

namespace {

// [0, HG_NOALLOC_MAX_INLETQ): inlet-Q conveyance totals; the last slot holds
// the error-flag word (int32 in its first 4 bytes).
static __device__ __align__(256) double g_noalloc_scratch[HG_NOALLOC_MAX_INLETQ + 1];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};   // device address of g_noalloc_scratch, per device

// Device address of the scratch array on `device` (which must be current).
// In host code the name g_noalloc_scratch is only a host-side stand-in, so the
// address is looked up once per device.
cudaError_t scratch_address(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int hg_rhs_device_noalloc(hg_ctx* ctx, const double* d_Q, double* d_dQ, int32_t* d_flags, void* stream) {
  if (!ctx || !d_Q || !d_dQ) {
    if (ctx) ctx->err = "hg_rhs_device_noalloc: null argument";
    return HG_ERR_ARG;
  }
  if (ctx->precision != HG_FP64) {
    ctx->err = "hg_rhs_device_noalloc: only FP64 contexts are supported";
    return HG_ERR_UNSUPPORTED;
  }
  // An inlet hydrograph would need the evaluation time (hg_rhs writes Q(t)
  // into the context's inlet-Q array first), and a state-dependent resistance
  // writes the context's own per-cell n and LayerNorm buffers before every
  // RHS: either would make this call read or write context memory that other
  // calls on the context's stream use, so both are refused.
  if (ctx->dm.nHydro > 0) {
    ctx->err = "hg_rhs_device_noalloc: the context has an inlet hydrograph; use hg_rhs (it takes the time t)";
    return HG_ERR_UNSUPPORTED;
  }
  if (ctx->dm.res.kind != hg::kResConstant) {
    ctx->err = "hg_rhs_device_noalloc: the context has a state-dependent resistance; use hg_rhs";
    return HG_ERR_UNSUPPORTED;
  }
  if (ctx->dm.nInlet > HG_NOALLOC_MAX_INLETQ) {
    ctx->err = "hg_rhs_device_noalloc: the mesh has " + std::to_string(ctx->dm.nInlet) +
               " inlet-Q boundaries; at most " + std::to_string(HG_NOALLOC_MAX_INLETQ) + " are supported";
    return HG_ERR_ARG;
  }
  if (ctx->device < 0 || ctx->device >= kMaxDevices) {
    ctx->err = "hg_rhs_device_noalloc: device index out of range";
    return HG_ERR_ARG;
  }
  (void)cudaGetLastError();   // an error left by earlier, unrelated work is not this call's
  cudaError_t e = cudaSetDevice(ctx->device);
  double* scratch = nullptr;
  if (e == cudaSuccess) e = scratch_address(ctx->device, &scratch);
  if (e != cudaSuccess) {
    ctx->err = std::string("hg_rhs_device_noalloc: set-up failed: ") + cudaGetErrorString(e);
    return HG_ERR_CUDA;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  int32_t* flags = reinterpret_cast<int32_t*>(scratch + HG_NOALLOC_MAX_INLETQ);
  hg::DevMesh m = ctx->dm;       // the context's read-only tables ...
  m.totalA = scratch;            // ... with the scratch in the static array
  hg::DevScalars s{};
  s.flags = flags;
  e = cudaMemsetAsync(flags, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) {
    hg::launch_inlet_total_f64(m, s, d_Q, st);
    hg::launch_stage_f64(m, s, hg::kModeRhs, d_Q, nullptr, d_dQ, false, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && d_flags) e = cudaMemcpyAsync(d_flags, flags, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) {
    ctx->err = std::string("hg_rhs_device_noalloc: ") + cudaGetErrorString(e);
    return HG_ERR_CUDA;
  }
  ctx->launches += 1 + (m.nInlet > 0 ? 1 : 0);   // no resistance kernels: refused above
  return HG_OK;
}
