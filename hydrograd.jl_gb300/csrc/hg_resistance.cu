// FP64 instantiations of the resistance kernels (hg_resistance.cuh).  This
// file is compiled without FMA contraction: the FP64 closures round as the
// oracle does.
#include "hg_resistance.cuh"

namespace hg {

int launch_ude_vjp_f64(const DevMesh& m, const AdjDev& a, const double* Q, double* out, cudaStream_t st) {
  return launch_ude_vjp<double, const double*, double>(m, a, Q, out, st);
}

int resistance_launches(const DevMesh& m) {
  if (m.res.kind == kResConstant || m.n == 0) return 0;
  return 1 + ((m.res.kind >= kResUdeManningH && m.res.overBatch) ? m.res.nHidden : 0);
}

int launch_resistance_f64(const DevMesh& m, const double* Q, cudaStream_t st) {
  return launch_resistance<double, const double*>(m, Q, st);
}

}  // namespace hg
