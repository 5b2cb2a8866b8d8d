// Fused step kernels (one cell per thread) for D2Q9 with BGK collision, in XLB's
// operation order (collision code 0), in pair form (code 2) and on stored deviations (code 3).
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_d2q9_bgk(const StepArgs& a, int sk, int compute, bool fullbc, bool diag, int form, cudaStream_t s) {
  return XLBG_BGK_FORM(launch_step_t, 0, a, sk, compute, fullbc, diag, s);
}
}  // namespace xlbg
