// Segmented two-cell step kernels for D3Q27 with the shifted 16-bit stores
// (one lattice per translation unit so the build parallelises).
#include "step_tma_seg.cuh"

namespace xlbg {
int launch_step_seg_d3q27(const StepArgs& a, int sk, int coll, bool fullbc, bool diag, int nseg, int rows, int* err,
                         cudaStream_t s) {
  return launch_seg_lattice<2>(a, sk, coll, fullbc, diag, nseg, rows, err, s);
}
}  // namespace xlbg
