// Adjoint kernels for D2Q9 (one lattice per translation unit so the build parallelises).
#include "adjoint.cuh"

namespace xlbg {
int launch_adjoint_d2q9(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s) {
  return launch_adjoint_t<0>(A, sk, compute, kbc, s);
}
}  // namespace xlbg
