// Adjoint kernels for D3Q27 (one lattice per translation unit so the build parallelises).
#include "adjoint.cuh"

namespace xlbg {
int launch_adjoint_d3q27(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s) {
  return launch_adjoint_t<2>(A, sk, compute, kbc, s);
}
}  // namespace xlbg
