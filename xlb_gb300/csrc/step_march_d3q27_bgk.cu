// Marching step kernels for D3Q27 with BGK collision, in XLB's operation order
// (collision code 0), in pair form (code 2) and on stored deviations (code 3).
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_march_d3q27_bgk(const StepArgs& a, int sk, int compute, bool fullbc, int form, int threads, int chunk,
                             cudaStream_t s) {
  return XLBG_BGK_FORM(launch_step_march_t, 2, a, sk, compute, fullbc, threads, chunk, s);
}
}  // namespace xlbg
