// TMA-staged step kernels for D3Q19 with the 16-bit stores (one lattice per
// translation unit so the build parallelises).
#include "step_tma_x2.cuh"

namespace xlbg {
int launch_step_tma_d3q19(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows, int box,
                       int* err, cudaStream_t s) {
  if (sk == SK_F16 && coll == 0) return launch_tma_t<1, SK_F16, 0>(map, a, fullbc, rows, box, err, s);
  if (sk == SK_F16S && coll == 2)
    return tma_x2_enabled() ? launch_tma_x2_t<1, SK_F16S>(map, a, fullbc, rows, box, err, s)
                            : launch_tma_t<1, SK_F16S, 2>(map, a, fullbc, rows, box, err, s);
  if (sk == SK_BF16S && coll == 2)
    return tma_x2_enabled() ? launch_tma_x2_t<1, SK_BF16S>(map, a, fullbc, rows, box, err, s)
                            : launch_tma_t<1, SK_BF16S, 2>(map, a, fullbc, rows, box, err, s);
  return -1;
}
}  // namespace xlbg
