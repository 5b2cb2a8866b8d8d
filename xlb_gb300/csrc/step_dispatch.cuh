// Launch of the fused step kernel for one (lattice, collision) pair.  Each
// step_*.cu translation unit instantiates one pair so the build parallelises.
#pragma once
#include <cuda_runtime.h>

#include "step_kernel.cuh"

namespace xlbg {

// Returns 0 on launch, -1 for an unsupported store/compute pair, or the CUDA error.
// Pick the instantiation of a BGK form (0, 2 or 3) at run time.
#define XLBG_BGK_FORM(FN, LAT, ...)                                                                  \
  (form == 4   ? FN<LAT, 4>(__VA_ARGS__)                                                                \
   : form == 3 ? FN<LAT, 3>(__VA_ARGS__)                                                                \
   : form == 2 ? FN<LAT, 2>(__VA_ARGS__)                                                                \
               : FN<LAT, 0>(__VA_ARGS__))
template <int LAT, int COLL>
int launch_step_t(const StepArgs& a, int sk, int compute, bool fullbc, bool diag, cudaStream_t s) {
  using L = Lattice<LAT>;
  const dim3 grid((unsigned)(a.n0 * a.n1), (unsigned)((a.n2 + kStepBlock - 1) / kStepBlock));
#define XLBG_LAUNCH(SKV, TV)                                                         \
  do {                                                                               \
    if (diag)                                                                        \
      step_kernel<L, SKV, TV, COLL, true, true><<<grid, kStepBlock, 0, s>>>(a);     \
    else if (fullbc)                                                                 \
      step_kernel<L, SKV, TV, COLL, true, false><<<grid, kStepBlock, 0, s>>>(a);    \
    else                                                                             \
      step_kernel<L, SKV, TV, COLL, false, false><<<grid, kStepBlock, 0, s>>>(a);   \
  } while (0)
  if constexpr (COLL == 4) {  // stochastic rounding: shifted 16-bit stores, FP32 compute only
    if (compute == 1) return -1;
    switch (sk) {
      case SK_F16S: XLBG_LAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_LAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  } else if constexpr (COLL == 3) {  // deviations: shifted stores or FP32, FP32 compute only
    if (compute == 1) return -1;
    switch (sk) {
      case SK_F32: XLBG_LAUNCH(SK_F32, float); break;
      case SK_F16S: XLBG_LAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_LAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  } else if (compute == 1) {
    switch (sk) {
      case SK_F64: XLBG_LAUNCH(SK_F64, double); break;
      case SK_F32: XLBG_LAUNCH(SK_F32, double); break;
      case SK_F16: XLBG_LAUNCH(SK_F16, double); break;
      default: return -1;
    }
  } else {
    switch (sk) {
      case SK_F32: XLBG_LAUNCH(SK_F32, float); break;
      case SK_F16: XLBG_LAUNCH(SK_F16, float); break;
      case SK_F16S: XLBG_LAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_LAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  }
#undef XLBG_LAUNCH
  return (int)cudaGetLastError();
}

// One marching-kernel instantiation family: offset width from a.wide, BC code from fullbc.
template <class L, int SKV, class TV, int COLL>
void launch_march_variant(const StepArgs& a, bool fullbc, dim3 grid, int threads, int chunk, cudaStream_t s) {
  if (a.diag_slots != nullptr) {  // the diagnostics step (always with the full BC code)
    if (a.wide)
      step_kernel_march<L, SKV, TV, COLL, true, long long, true><<<grid, threads, 0, s>>>(a, chunk);
    else
      step_kernel_march<L, SKV, TV, COLL, true, unsigned, true><<<grid, threads, 0, s>>>(a, chunk);
  } else if (a.wide) {
    if (fullbc)
      step_kernel_march<L, SKV, TV, COLL, true, long long><<<grid, threads, 0, s>>>(a, chunk);
    else
      step_kernel_march<L, SKV, TV, COLL, false, long long><<<grid, threads, 0, s>>>(a, chunk);
  } else {
    if (fullbc)
      step_kernel_march<L, SKV, TV, COLL, true, unsigned><<<grid, threads, 0, s>>>(a, chunk);
    else
      step_kernel_march<L, SKV, TV, COLL, false, unsigned><<<grid, threads, 0, s>>>(a, chunk);
  }
}

// Marching kernel; `threads` per block (multiple of 32), `chunk` rows of axis 1 per thread.
template <int LAT, int COLL>
int launch_step_march_t(const StepArgs& a, int sk, int compute, bool fullbc, int threads, int chunk, cudaStream_t s) {
  using L = Lattice<LAT>;
  const int zblocks = (a.n2 + threads - 1) / threads;
  const dim3 grid((unsigned)(a.n0 * zblocks), (unsigned)((a.n1 + chunk - 1) / chunk));
#define XLBG_MLAUNCH(SKV, TV) launch_march_variant<L, SKV, TV, COLL>(a, fullbc, grid, threads, chunk, s)
  if constexpr (COLL == 4) {  // stochastic rounding: shifted 16-bit stores, FP32 compute only
    if (compute == 1) return -1;
    switch (sk) {
      case SK_F16S: XLBG_MLAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_MLAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  } else if constexpr (COLL == 3) {  // deviations: shifted stores or FP32, FP32 compute only
    if (compute == 1) return -1;
    switch (sk) {
      case SK_F32: XLBG_MLAUNCH(SK_F32, float); break;
      case SK_F16S: XLBG_MLAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_MLAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  } else if (compute == 1) {
    switch (sk) {
      case SK_F64: XLBG_MLAUNCH(SK_F64, double); break;
      case SK_F32: XLBG_MLAUNCH(SK_F32, double); break;
      case SK_F16: XLBG_MLAUNCH(SK_F16, double); break;
      default: return -1;
    }
  } else {
    switch (sk) {
      case SK_F32: XLBG_MLAUNCH(SK_F32, float); break;
      case SK_F16: XLBG_MLAUNCH(SK_F16, float); break;
      case SK_F16S: XLBG_MLAUNCH(SK_F16S, float); break;
      case SK_BF16S: XLBG_MLAUNCH(SK_BF16S, float); break;
      default: return -1;
    }
  }
#undef XLBG_MLAUNCH
  return (int)cudaGetLastError();
}

// BGK launchers take the BGK form: 0 (XLB order), 2 (pair form) or 3 (stored deviations).
int launch_step_march_d2q9_bgk(const StepArgs&, int, int, bool, int, int, int, cudaStream_t);
int launch_step_march_d2q9_kbc(const StepArgs&, int, int, bool, int, int, cudaStream_t);
int launch_step_march_d3q19_bgk(const StepArgs&, int, int, bool, int, int, int, cudaStream_t);
int launch_step_march_d3q27_bgk(const StepArgs&, int, int, bool, int, int, int, cudaStream_t);
int launch_step_march_d3q27_kbc(const StepArgs&, int, int, bool, int, int, cudaStream_t);

int launch_step_d2q9_bgk(const StepArgs&, int, int, bool, bool, int, cudaStream_t);
int launch_step_d2q9_kbc(const StepArgs&, int, int, bool, bool, cudaStream_t);
int launch_step_d3q19_bgk(const StepArgs&, int, int, bool, bool, int, cudaStream_t);
int launch_step_d3q27_bgk(const StepArgs&, int, int, bool, bool, int, cudaStream_t);
int launch_step_d3q27_kbc(const StepArgs&, int, int, bool, bool, cudaStream_t);

}  // namespace xlbg
