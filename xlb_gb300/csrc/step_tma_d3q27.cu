// TMA-staged step kernels for D3Q27 with the 16-bit stores (one lattice per
// translation unit so the build parallelises).
#include "step_tma.cuh"

namespace xlbg {
int launch_step_tma_d3q27(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows, int box,
                       int* err, cudaStream_t s) {
  if (sk == SK_F16 && coll == 0) return launch_tma_t<2, SK_F16, 0>(map, a, fullbc, rows, box, err, s);
  // one cell per consumer: the two-cell kernel's 27 packed populations spill
  if (sk == SK_F16S && coll == 2) return launch_tma_t<2, SK_F16S, 2>(map, a, fullbc, rows, box, err, s);
  if (sk == SK_BF16S && coll == 2) return launch_tma_t<2, SK_BF16S, 2>(map, a, fullbc, rows, box, err, s);
  return -1;
}
}  // namespace xlbg
