// Fused step kernels (one cell per thread) for D2Q9 with BGK collision, in XLB's
// operation order (collision code 0) and in pair form (collision code 2).
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_d2q9_bgk(const StepArgs& a, int sk, int compute, bool fullbc, bool diag, bool pair, cudaStream_t s) {
  return pair ? launch_step_t<0, 2>(a, sk, compute, fullbc, diag, s) : launch_step_t<0, 0>(a, sk, compute, fullbc, diag, s);
}
}  // namespace xlbg
