// Fused step kernels for D3Q19 with BGK collision.
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_d3q19_bgk(const StepArgs& a, int sk, int compute, bool fullbc, bool diag, cudaStream_t s) {
  return launch_step_t<1, 0>(a, sk, compute, fullbc, diag, s);
}
}  // namespace xlbg
