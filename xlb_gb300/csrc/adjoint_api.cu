// C ABI of the differentiation path: forward recording of a segment of states
// and the reverse (adjoint) sweep over it.  Declarations and contracts are in
// include/xlbg.h.
#include <cuda_runtime.h>

#include "../../include/xlbg.h"
#include "adjoint.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int store_bytes(int sk);
int check_ptr(const void* p, int align, const char* name);
int check_step_args(const xlbg_desc* d, const void* f0, const void* f1, const uint8_t* bc_mask, const uint32_t* miss,
                    const int64_t* rec_cells, int64_t n_rec, const void* rec_scratch);
int fill_step_args(const xlbg_desc* d, const void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
                   double omega, StepArgs& a);
int launch_main(const xlbg_desc* d, const StepArgs& a, bool diag, cudaStream_t s);

static bool has_aux_bc(const xlbg_desc* d) {
  for (int b = 0; b < d->nbc; ++b)
    if (d->bc[b].kind >= XLBG_BC_ZOUHE_VELOCITY && d->bc[b].kind <= XLBG_BC_REGULARIZED_PRESSURE) return true;
  return false;
}

static long long state_bytes(const xlbg_desc* d) {
  const int q = d->lattice == XLBG_D2Q9 ? 9 : (d->lattice == XLBG_D3Q19 ? 19 : 27);
  return (long long)q * d->nx * d->ny * d->nz * store_bytes(d->store);
}

static int check_segment(const xlbg_desc* d, const void* states, int32_t n_steps, const uint8_t* bc_mask,
                         const uint32_t* miss, const void* aux) {
  // a state pair that is certainly distinct, so check_step_args validates the rest
  const char* s0 = static_cast<const char*>(states);
  int e = check_step_args(d, states, s0 + state_bytes(d), bc_mask, miss, nullptr, 0, nullptr);
  if (e) return e;
  if (n_steps < 0) return fail(XLBG_ERR_ARG, "n_steps < 0");
  if (has_aux_bc(d) && (e = check_ptr(aux, store_bytes(d->store), "aux"))) return e;
  return XLBG_OK;
}

static int adjoint_dispatch(const xlbg_desc* d, const AdjArgs& A, cudaStream_t s) {
  const bool kbc = d->collision == XLBG_KBC;
  const int r = d->lattice == XLBG_D2Q9    ? launch_adjoint_d2q9(A, d->store, d->compute, kbc, s)
                : d->lattice == XLBG_D3Q19 ? launch_adjoint_d3q19(A, d->store, d->compute, kbc, s)
                                           : launch_adjoint_d3q27(A, d->store, d->compute, kbc, s);
  if (r < 0)
    return fail(XLBG_ERR_UNSUPPORTED, "adjoint supports FP32 store with FP32 or FP64 compute and FP64/FP64 only");
  if (r) return fail(XLBG_ERR_CUDA, "adjoint launch: %s", cudaGetErrorString((cudaError_t)r));
  return XLBG_OK;
}

}  // namespace xlbg

using namespace xlbg;

extern "C" {

int xlbg_forward_segment(const xlbg_desc* desc, void* states, int32_t n_steps, const uint8_t* bc_mask,
                         const uint32_t* miss_bits, const void* aux, double omega, void* stream) {
  int e = check_segment(desc, states, n_steps, bc_mask, miss_bits, aux);
  if (e) return e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long sb = state_bytes(desc);
  char* base = static_cast<char*>(states);
  for (int j = 0; j < n_steps; ++j) {
    StepArgs a;
    fill_step_args(desc, base + j * sb, base + (j + 1) * sb, bc_mask, miss_bits, omega, a);
    a.aux = aux;
    if ((e = launch_main(desc, a, false, s))) return e;
  }
  return XLBG_OK;
}

int xlbg_adjoint_segment(const xlbg_desc* desc, const void* states, int32_t n_steps, const uint8_t* bc_mask,
                         const uint32_t* miss_bits, const void* aux, const int64_t* bc_cells, int64_t n_bc,
                         void* lam_a, void* lam_b, void* aux_grad, double omega, void* stream) {
  int e = check_segment(desc, states, n_steps, bc_mask, miss_bits, aux);
  if (e) return e;
  const int cb = desc->compute == XLBG_COMPUTE_F64 ? 8 : 4;
  if ((e = check_ptr(lam_a, cb, "lam_a"))) return e;
  if ((e = check_ptr(lam_b, cb, "lam_b"))) return e;
  if (lam_a == lam_b) return fail(XLBG_ERR_ARG, "lam_a and lam_b must be distinct buffers");
  if (n_bc < 0) return fail(XLBG_ERR_ARG, "n_bc < 0");
  if (n_bc > 0) {
    if ((e = check_ptr(bc_cells, 8, "bc_cells"))) return e;
    if ((e = check_ptr(aux_grad, cb, "aux_grad"))) return e;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long sb = state_bytes(desc);
  const char* base = static_cast<const char*>(states);
  for (int k = 0; k < n_steps; ++k) {
    const int j = n_steps - 1 - k;  // forward step j: state j -> state j + 1
    AdjArgs A;
    fill_step_args(desc, base + j * sb, nullptr, bc_mask, miss_bits, omega, A.s);
    A.s.aux = aux;
    A.lam_out = (k % 2 == 0) ? lam_a : lam_b;
    A.lam_in = (k % 2 == 0) ? lam_b : lam_a;
    A.bc_cells = reinterpret_cast<const long long*>(bc_cells);
    A.n_bc = n_bc;
    A.aux_grad = aux_grad;
    if ((e = adjoint_dispatch(desc, A, s))) return e;
  }
  return XLBG_OK;
}

}  // extern "C"
