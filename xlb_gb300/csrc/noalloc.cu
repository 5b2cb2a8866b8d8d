// xlbg_step_diag_noalloc: the diagnostics step without any caller-provided or
// library-allocated scratch.
//
// Some callers cannot allocate device memory around a step: hosts that own
// the whole device heap through their own pool and give a library only the
// buffers it reads and writes (embedded solvers with a fixed memory budget,
// plug-in hosts), and loops that must not call cudaMalloc / cudaFree because
// those calls can synchronise the whole device.  xlbg_step_diag needs two
// scratch buffers (the block partial sums of the FP64 reductions and the
// aux-recovery staging); this variant keeps both in file-scope __device__
// arrays of fixed size, so a call touches only the caller's inputs and outputs
// plus that static storage.
//
// Every GPU that loads libxlbg.so holds these arrays (about 4 MiB) until the
// process exits.  All calls on a device share them: calls whose GPU work can
// overlap (different streams without ordering, or several host threads)
// race on the scratch and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/xlbg.h"
#include "ctx.cuh"
#include "step_dispatch.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int store_bytes(int sk);
int check_ptr(const void* p, int align, const char* name);
int check_step_args(const xlbg_desc* d, const void* f0, const void* f1, const uint8_t* bc_mask, const uint32_t* miss,
                    const int64_t* rec_cells, int64_t n_rec, const void* rec_scratch);
int one_step(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
             const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, bool diag, int force_id,
             double* slots, double* out, cudaStream_t s, int timestep);

// Block partial sums of the diagnostics reduction (zeroed at the start of each call).
static __device__ __align__(256) double g_noalloc_diag_slots[XLBG_DIAG_SLOTS * 4];
// Aux-recovery staging: n_rec * Q * store-bytes must fit.
static __device__ __align__(256) unsigned char g_noalloc_rec_scratch[XLBG_NOALLOC_REC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
struct NoallocPtrs {
  double* slots = nullptr;
  void* rec = nullptr;
  void* ctx = nullptr;  // context the addresses belong to
  bool ready = false;
};
std::mutex g_noalloc_mu;
NoallocPtrs g_noalloc_ptrs[kMaxDevices];

// Device addresses of the static arrays for the current device.  In host code
// the array names are host-side stand-ins, never device addresses; only
// cudaGetSymbolAddress yields the real ones.  They are looked up on the first
// call on a device (with that device current) and again whenever the device's
// context has changed since (cudaDeviceReset gives it a new one).
int noalloc_pointers(NoallocPtrs& out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(XLBG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(XLBG_ERR_ARG, "device ordinal %d outside 0..%d", dev, kMaxDevices - 1);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocPtrs& p = g_noalloc_ptrs[dev];
  void* ctx = current_context();
  if (!p.ready || ctx == nullptr || ctx != p.ctx) {
    void* slots = nullptr;
    void* rec = nullptr;
    e = cudaGetSymbolAddress(&slots, g_noalloc_diag_slots);
    if (e != cudaSuccess) return fail(XLBG_ERR_CUDA, "cudaGetSymbolAddress(diag slots): %s", cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&rec, g_noalloc_rec_scratch);
    if (e != cudaSuccess) return fail(XLBG_ERR_CUDA, "cudaGetSymbolAddress(recovery scratch): %s", cudaGetErrorString(e));
    p.slots = static_cast<double*>(slots);
    p.rec = rec;
    p.ctx = current_context();  // the lookup made the primary context current if it was not
    p.ready = true;
  }
  out = p;
  return XLBG_OK;
}
}  // namespace

}  // namespace xlbg

using namespace xlbg;

extern "C" int xlbg_step_diag_noalloc(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask,
                                      const uint32_t* miss, const int64_t* rec_cells, int64_t n_rec, double omega,
                                      int32_t timestep, int32_t force_id, double* diag, void* stream) {
  NoallocPtrs p;
  int e;
  if ((e = noalloc_pointers(p))) return e;
  if ((e = check_step_args(d, f0, f1, bc_mask, miss, rec_cells, n_rec, p.rec))) return e;
  if ((e = check_ptr(diag, 8, "diag"))) return e;
  const int q = d->lattice == XLBG_D2Q9 ? 9 : (d->lattice == XLBG_D3Q19 ? 19 : 27);
  // compared by division: n_rec * q * bytes could overflow for a bogus n_rec
  const long long per_cell = (long long)q * store_bytes(d->store);
  if (n_rec > (long long)XLBG_NOALLOC_REC_SCRATCH_BYTES / per_cell)
    return fail(XLBG_ERR_ARG,
                "xlbg_step_diag_noalloc: %lld recovery cells x %d directions x %d bytes exceeds the "
                "%u-byte static scratch (at most %lld cells); use xlbg_step_diag with caller scratch",
                (long long)n_rec, q, store_bytes(d->store), (unsigned)XLBG_NOALLOC_REC_SCRATCH_BYTES,
                (long long)XLBG_NOALLOC_REC_SCRATCH_BYTES / per_cell);
  cudaStream_t s = (cudaStream_t)stream;
  // The slots keep the previous call's contents; the reduction needs them zero.
  cudaError_t ce = cudaMemsetAsync(p.slots, 0, sizeof(double) * XLBG_DIAG_SLOTS * 4, s);
  if (ce != cudaSuccess) return fail(XLBG_ERR_CUDA, "clearing the diagnostics slots: %s", cudaGetErrorString(ce));
  return one_step(d, f0, f1, bc_mask, miss, rec_cells, n_rec, p.rec, omega, true, force_id, p.slots, diag, s,
                  timestep);
}
