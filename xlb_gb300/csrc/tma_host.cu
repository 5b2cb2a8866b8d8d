// Host side of the TMA-staged step (step_tma.cuh): applicability, tensor-map
// encoding, the device error flag of the bounded waits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/xlbg.h"
#include "ctx.cuh"
#include "step_tma.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);

// Set by a TMA-staged block whose stage did not complete within its bounded wait.
__device__ int g_tma_fault = 0;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

std::mutex g_mu;
int* g_fault_ptr[64] = {nullptr};
void* g_fault_ctx[64] = {nullptr};

// Device address of g_tma_fault on the current device, looked up again when the
// device's context has changed (after cudaDeviceReset).
int* fault_ptr() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  void* ctx = current_context();
  if (!g_fault_ptr[dev] || ctx == nullptr || ctx != g_fault_ctx[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tma_fault) != cudaSuccess) return nullptr;
    g_fault_ptr[dev] = static_cast<int*>(p);
    g_fault_ctx[dev] = current_context();
  }
  return g_fault_ptr[dev];
}

}  // namespace

// Launches the TMA-staged step when it applies: FP32 compute, a contiguous
// axis of at least 8 cells that is a multiple of 8, fewer than 2^31 cells and a
// 16-byte aligned f0.  The shifted 16-bit stores with BGK on their deviations
// (codes 3 and 4) take the segmented two-cell kernel (any row length, also the
// diagnostics step); raw FP16 with XLB-order BGK (not the diagnostics step) and
// FP32 D3Q27 KBC (also with diagnostics) stage whole rows of at most 512 cells.  Boundary paths index planes in 32 bits when Q * cells <
// 2^32, else in 64 bits (as do the calls made with a.wide set).  Returns 1 when
// it does not apply (the caller uses the marching kernel), else the status.
int try_launch_tma(const xlbg_desc* d, const StepArgs& a, bool fullbc, bool diag, cudaStream_t s) {
  if (d->compute != XLBG_COMPUTE_F32) return 1;
  const int sk = d->store;
  const int coll = d->collision;
  const bool pair = (sk == SK_F16S || sk == SK_BF16S) && (coll == XLBG_BGK_SHIFTED || coll == XLBG_BGK_SHIFTED_SR);
  const bool raw16 = sk == SK_F16 && coll == XLBG_BGK;
  // FP32 D3Q27 KBC: the compute-heavy sphere-channel step, also with diagnostics
  const bool kbc32 = sk == SK_F32 && coll == XLBG_KBC && d->lattice == XLBG_D3Q27;
  if (!(pair || (raw16 && !diag) || kbc32)) return 1;
  const int q = d->lattice == XLBG_D2Q9 ? 9 : (d->lattice == XLBG_D3Q19 ? 19 : 27);
  const int eb = kbc32 ? 4 : 2;
  const bool seg = pair;
  // rows of 16-byte multiples; whole rows of at most 512 cells (a 1024-cell stage
  // leaves one CTA a SM: raw FP16 at 1024 x 1024 x 768 ran at 36 GLUPS there
  // against 41 on the marching kernel)
  if (a.n2 < 8 || (a.n2 * eb) % 16 != 0) return 1;
  if (!seg && a.n2 > 512) return 1;
  if (a.ncell >= 0x7fffffffLL) return 1;
  if (reinterpret_cast<uintptr_t>(a.f0) % 16 != 0) return 1;
  // the two-cell kernel of collision codes 3 and 4 loads ids and stores outputs in pairs
  if (pair && (reinterpret_cast<uintptr_t>(a.bc_mask) % 2 != 0 || reinterpret_cast<uintptr_t>(a.f1) % 4 != 0))
    return 1;
  int* err = fault_ptr();
  if (!err) return 1;

  if (seg) {
    // segments: rows of axis 1 per block for about 32 resident waves of four
    // blocks a SM over 152 SMs, at most 96 rows (D3Q19 FP16S, rows per block:
    // 512^3 54 -> 82.6, 27 -> 84.4, 14 -> 83.5 GLUPS; 1024 x 1024 x 768 162 ->
    // 82.0, 81 -> 83.4; the last wave's imbalance against each block's ring fill)
    const int nseg = (a.n2 + kSeg - 1) / kSeg;
    const long long target = 152LL * 4 * 32;
    long long rows = ((long long)a.n0 * nseg * a.n1 + target - 1) / target;
    if (rows > 96) rows = 96;
    if (rows < 1) rows = 1;
    if (rows > a.n1) rows = a.n1;
    const long long bands = (a.n1 + rows - 1) / rows;
    rows = (a.n1 + bands - 1) / bands;  // even bands
    int r;
    if (d->lattice == XLBG_D2Q9)
      r = launch_step_seg_d2q9(a, sk, coll, fullbc, diag, nseg, (int)rows, err, s);
    else if (d->lattice == XLBG_D3Q19)
      r = launch_step_seg_d3q19(a, sk, coll, fullbc, diag, nseg, (int)rows, err, s);
    else
      r = launch_step_seg_d3q27(a, sk, coll, fullbc, diag, nseg, (int)rows, err, s);
    if (r < 0) return 1;
    if (r) return fail(XLBG_ERR_CUDA, "segmented step kernel launch: %s", cudaGetErrorString((cudaError_t)r));
    return XLBG_OK;
  }

  EncodeTiledFn enc = encode_fn();
  if (!enc) return 1;

  const int box = a.n2 < kTmaBox ? a.n2 : kTmaBox;
  CUtensorMap map;
  const cuuint64_t dims[4] = {(cuuint64_t)a.n2, (cuuint64_t)a.n1, (cuuint64_t)a.n0, (cuuint64_t)q};
  const cuuint64_t strides[3] = {(cuuint64_t)a.n2 * eb, (cuuint64_t)a.n1 * a.n2 * eb, (cuuint64_t)a.ncell * eb};
  const cuuint32_t boxdim[4] = {(cuuint32_t)box, 1, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  if (enc(&map, eb == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 4, const_cast<void*>(a.f0),
          dims, strides, boxdim, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 1;

  // rows of axis 1 per CTA: about 32 resident waves of CTAs over 152 SMs (FP32
  // D3Q27 KBC on the 768 x 192 x 192 sphere channel, developed flow: 16 waves
  // 16.2, 32 waves 16.9, 64 waves 16.8 GLUPS)
  const int cps = eb == 4 ? (a.n2 <= 256 ? 2 : 1) : (a.n2 <= 256 ? 4 : (a.n2 <= 512 ? 2 : 1));
  const long long target = 152LL * cps * 32;
  long long rows = ((long long)a.n0 * a.n1 + target - 1) / target;
  if (rows < 1) rows = 1;
  if (rows > a.n1) rows = a.n1;

  int r;
  if (kbc32)
    r = launch_step_tma_d3q27_kbc32(map, a, fullbc, (int)rows, box, err, s);
  else if (d->lattice == XLBG_D2Q9)
    r = launch_step_tma_d2q9(map, a, sk, coll, fullbc, (int)rows, box, err, s);
  else if (d->lattice == XLBG_D3Q19)
    r = launch_step_tma_d3q19(map, a, sk, coll, fullbc, (int)rows, box, err, s);
  else
    r = launch_step_tma_d3q27(map, a, sk, coll, fullbc, (int)rows, box, err, s);
  if (r < 0) return 1;
  if (r) return fail(XLBG_ERR_CUDA, "TMA step kernel launch: %s", cudaGetErrorString((cudaError_t)r));
  return XLBG_OK;
}

}  // namespace xlbg

extern "C" int xlbg_device_faults(int reset) {
  using namespace xlbg;
  int* p = fault_ptr();
  if (!p) return -XLBG_ERR_CUDA;
  int v = 0;
  if (cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -XLBG_ERR_CUDA;
  if (reset && v) {
    const int zero = 0;
    if (cudaMemcpy(p, &zero, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) return -XLBG_ERR_CUDA;
  }
  return v;
}
