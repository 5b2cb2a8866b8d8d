// TMA-staged step kernels for D3Q27 with raw FP16 stores (one lattice per
// translation unit so the build parallelises).
#include "step_tma.cuh"

namespace xlbg {
int launch_step_tma_d3q27(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows, int box,
                       int* err, cudaStream_t s) {
  return launch_tma_lattice<2>(map, a, sk, coll, fullbc, rows, box, err, s);
}
}  // namespace xlbg
