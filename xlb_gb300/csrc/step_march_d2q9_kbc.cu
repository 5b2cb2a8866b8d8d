// Marching step kernels for D2Q9 with KBC collision.
#include "step_dispatch.cuh"

namespace xlbg {
int launch_step_march_d2q9_kbc(const StepArgs& a, int sk, int compute, bool fullbc, int threads, int chunk, cudaStream_t s) {
  return launch_step_march_t<0, 1>(a, sk, compute, fullbc, threads, chunk, s);
}
}  // namespace xlbg
