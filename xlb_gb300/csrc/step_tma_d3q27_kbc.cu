// TMA-staged step kernels for D3Q27 KBC with FP32 storage, plain and with the
// fused diagnostics (its own translation unit: the KBC instantiations are the
// largest in the library).
#include "step_tma.cuh"

namespace xlbg {
int launch_step_tma_d3q27_kbc32(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                                cudaStream_t s) {
  return launch_tma_t<2, SK_F32, 1, true>(map, a, fullbc, rows, box, err, s);
}
}  // namespace xlbg
