// Marching step kernels for D3Q19 with BGK collision, in XLB's operation order
// (collision code 0) and in pair form (collision code 2).
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_march_d3q19_bgk(const StepArgs& a, int sk, int compute, bool fullbc, bool pair, int threads, int chunk,
                             cudaStream_t s) {
  return pair ? launch_step_march_t<1, 2>(a, sk, compute, fullbc, threads, chunk, s)
              : launch_step_march_t<1, 0>(a, sk, compute, fullbc, threads, chunk, s);
}
}  // namespace xlbg
