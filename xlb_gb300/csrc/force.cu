// xlbg_momentum_transfer: the momentum-exchange force on one no-slip BC as a
// standalone operator (xlb/operator/force/momentum_transfer.py:92-176).
//
// XLB launches one thread per cell: at an "edge" cell (bc_mask == the BC's id
// and the rest direction not missing, :126-131) it pulls, applies the no-slip
// functional and adds, for every missing direction l,
// phi_l = f0[opp l] + f_post_stream[l] signed by c[opp l] to a per-thread vector
// in the compute type (:144-158), then atomically into one vector.  Both no-slip
// functionals give f_post_stream[l] = f0[opp l] at the cell for a missing l
// (halfway: the own-cell value of the opposite slot; fullway: f_pre[opp l]), so
// phi_l = 2 f0[opp l].
//
// Here each thread walks cells with a grid stride, reading bc_mask one byte a
// cell and, at edge cells only, the Q missing flags (XLB's bool form) and the Q
// own-cell populations.  Per-cell sums stay in the compute type as in XLB; the
// sums over cells are FP64 (warp shuffles, one atomic per block into a slot of
// the caller's slot array, then one finalising block), where XLB adds FP32
// atomics in launch order.
#include <cuda_runtime.h>

#include "../../include/xlbg.h"
#include "step_kernel.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int store_bytes(int sk);
int check_ptr(const void* p, int align, const char* name);
int check_desc_public(const xlbg_desc* d);
int launch_diag_finalize(double* slots, double* out, cudaStream_t s);

namespace {

template <class L, int SK, class T>
__global__ void __launch_bounds__(kStepBlock) momentum_transfer_kernel(const typename Store<SK, T>::Bits* __restrict__ f0,
                                                                       const uint8_t* __restrict__ bc_mask,
                                                                       const uint8_t* __restrict__ missing, long long n,
                                                                       int bc_id, double* __restrict__ slots) {
  using St = Store<SK, T>;
  constexpr int Q = L::Q;
  double acc[3] = {0.0, 0.0, 0.0};
  const uint8_t id = (uint8_t)bc_id;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    if (bc_mask[c] != id || missing[c] != 0) continue;  // edge: the BC's id, rest direction present
    T m[L::D];
#pragma unroll
    for (int d = 0; d < L::D; ++d) m[d] = T(0);
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      if (missing[(long long)l * n + c]) {
        const T v = St::dec(f0[(long long)opp<L>(l) * n + c], T(weight<L>(opp<L>(l))));
        const T phi = v + v;
#pragma unroll
        for (int d = 0; d < L::D; ++d) {
          if (L::c(opp<L>(l), d) == 1) m[d] = m[d] + phi;
          if (L::c(opp<L>(l), d) == -1) m[d] = m[d] - phi;
        }
      }
    }
#pragma unroll
    for (int d = 0; d < L::D; ++d) acc[d] += (double)m[d];
  }
  reduce_diag(0.0, acc, slots);
}

template <class L, int SK, class T>
int mt_launch(long long n, const void* f0, const uint8_t* bc_mask, const uint8_t* missing, int bc_id, double* slots,
              double* out, cudaStream_t s) {
  long long blocks = (n + kStepBlock - 1) / kStepBlock;
  if (blocks > 152LL * 8) blocks = 152LL * 8;  // grid stride: eight blocks per SM of a 152-SM GB300
  if (blocks < 1) blocks = 1;
  momentum_transfer_kernel<L, SK, T><<<(unsigned)blocks, kStepBlock, 0, s>>>(
      static_cast<const typename Store<SK, T>::Bits*>(f0), bc_mask, missing, n, bc_id, slots);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = (cudaError_t)launch_diag_finalize(slots, out, s);
  return e == cudaSuccess ? XLBG_OK : fail(XLBG_ERR_CUDA, "momentum transfer launch: %s", cudaGetErrorString(e));
}

template <class L>
int mt_by_store(const xlbg_desc* d, long long n, const void* f0, const uint8_t* bc_mask, const uint8_t* missing,
                int bc_id, double* slots, double* out, cudaStream_t s) {
  const int sk = d->store;
  if (d->compute == XLBG_COMPUTE_F64) {
    if (sk == SK_F64) return mt_launch<L, SK_F64, double>(n, f0, bc_mask, missing, bc_id, slots, out, s);
    if (sk == SK_F32) return mt_launch<L, SK_F32, double>(n, f0, bc_mask, missing, bc_id, slots, out, s);
    if (sk == SK_F16) return mt_launch<L, SK_F16, double>(n, f0, bc_mask, missing, bc_id, slots, out, s);
  } else {
    if (sk == SK_F32) return mt_launch<L, SK_F32, float>(n, f0, bc_mask, missing, bc_id, slots, out, s);
    if (sk == SK_F16) return mt_launch<L, SK_F16, float>(n, f0, bc_mask, missing, bc_id, slots, out, s);
    if (sk == SK_F16S) return mt_launch<L, SK_F16S, float>(n, f0, bc_mask, missing, bc_id, slots, out, s);
    if (sk == SK_BF16S) return mt_launch<L, SK_BF16S, float>(n, f0, bc_mask, missing, bc_id, slots, out, s);
  }
  return fail(XLBG_ERR_UNSUPPORTED, "store/compute pair not supported");
}

}  // namespace
}  // namespace xlbg

using namespace xlbg;

extern "C" int xlbg_momentum_transfer(const xlbg_desc* d, const void* f0, const uint8_t* bc_mask,
                                      const uint8_t* missing_mask, int32_t bc_id, double* diag_slots, double* force,
                                      void* stream) {
  int e;
  if ((e = check_desc_public(d))) return e;
  if ((e = check_ptr(f0, store_bytes(d->store), "f0"))) return e;
  if ((e = check_ptr(bc_mask, 1, "bc_mask"))) return e;
  if ((e = check_ptr(missing_mask, 1, "missing_mask"))) return e;
  if ((e = check_ptr(diag_slots, 8, "diag_slots"))) return e;
  if ((e = check_ptr(force, 8, "force"))) return e;
  if (bc_id < 1 || bc_id > 254) return fail(XLBG_ERR_ARG, "bc id %d outside 1..254", bc_id);
  const long long n = d->nx * d->ny * d->nz;
  cudaStream_t s = (cudaStream_t)stream;
  if (d->lattice == XLBG_D2Q9) return mt_by_store<Lattice<0>>(d, n, f0, bc_mask, missing_mask, bc_id, diag_slots, force, s);
  if (d->lattice == XLBG_D3Q19) return mt_by_store<Lattice<1>>(d, n, f0, bc_mask, missing_mask, bc_id, diag_slots, force, s);
  return mt_by_store<Lattice<2>>(d, n, f0, bc_mask, missing_mask, bc_id, diag_slots, force, s);
}
