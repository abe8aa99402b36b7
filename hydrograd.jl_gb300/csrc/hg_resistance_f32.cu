// FP32 instantiations of the resistance kernels (hg_resistance.cuh) for the
// FP32-compensated path.  Compiled with FMA contraction (the FP64 unit is not).
#include "hg_resistance.cuh"

namespace hg {

int launch_ude_vjp_f32(const DevMesh& m, const AdjDev& a, StateF32 Q, float* out, cudaStream_t st) {
  return launch_ude_vjp<float, StateF32, float>(m, a, Q, out, st);
}

int launch_resistance_f32(const DevMesh& m, StateF32 X, cudaStream_t st) {
  return launch_resistance<float, StateF32>(m, X, st);
}

}  // namespace hg
