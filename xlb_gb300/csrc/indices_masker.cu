// Indices boundary masker: bc_mask / missing_mask from one BC's index list,
// the per-index work of XLB's Warp IndicesBoundaryMasker kernel
// (xlb/operator/boundary_masker/indices_boundary_masker.py:114-156).
//
// One thread per index.  An index outside the domain is skipped.  Otherwise
// the cell gets the BC id; for every direction l, when the pull source
// index - c_l is outside the domain the cell's direction l is missing, and
// otherwise, for a BC that needs padding and an index strictly inside the
// domain (are_indices_in_interior, :29-40), the push neighbour index + c_l gets
// the BC id and its direction l is missing (l = 0 marks the cell itself).
//
// XLB launches one kernel over the indices of all BCs, so a cell that two BCs
// touch gets whichever id is stored last.  Here the host calls this once per
// BC in list order: within one launch every store to an address writes the
// same value (the BC's id, or true), so the later BC's id wins and the result
// does not depend on thread order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xlbg.h"
#include "lattice.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int check_ptr(const void* p, int align, const char* name);

namespace {

template <class L>
__global__ void indices_mask(const int64_t* __restrict__ idx, long long n, int bc_id, int needs_padding, int nx,
                             int ny, int nz, uint8_t* __restrict__ bc_mask, uint8_t* __restrict__ missing) {
  const long long ii = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= n) return;
  const long long x = idx[ii], y = idx[n + ii], z = idx[2 * n + ii];
  if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return;
  const long long ncell = (long long)nx * ny * nz;
  const long long cell = (x * ny + y) * nz + z;
  // interior over the lattice's d axes (a 2D grid has nz == 1 and z == 0)
  const bool interior = needs_padding && x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && (L::D == 2 || (z > 0 && z < nz - 1));
  bc_mask[cell] = (uint8_t)bc_id;
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    const int cx = L::c(l, 0), cy = L::c(l, 1), cz = L::D == 3 ? L::c(l, 2) : 0;
    const long long px = x - cx, py = y - cy, pz = z - cz;
    if (px < 0 || px >= nx || py < 0 || py >= ny || pz < 0 || pz >= nz) {
      missing[l * ncell + cell] = 1;
    } else if (interior) {
      const long long push = ((x + cx) * ny + (y + cy)) * nz + (z + cz);
      missing[l * ncell + push] = 1;
      bc_mask[push] = (uint8_t)bc_id;
    }
  }
}

}  // namespace
}  // namespace xlbg

using namespace xlbg;

extern "C" int xlbg_indices_mask(const xlbg_desc* desc, const int64_t* indices, int64_t n, int32_t bc_id,
                                 int32_t needs_padding, uint8_t* bc_mask, uint8_t* missing_mask, void* stream) {
  if (!desc || desc->abi_version != XLBG_ABI_VERSION) return fail(XLBG_ERR_ARG, "bad descriptor");
  if (desc->lattice < XLBG_D2Q9 || desc->lattice > XLBG_D3Q27) return fail(XLBG_ERR_ARG, "bad lattice");
  if (n < 0 || bc_id < 1 || bc_id > 254) return fail(XLBG_ERR_ARG, "bad n or bc_id");
  if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1 || desc->nx > INT32_MAX || desc->ny > INT32_MAX ||
      desc->nz > INT32_MAX || (desc->lattice == XLBG_D2Q9 && desc->nz != 1))
    return fail(XLBG_ERR_ARG, "bad grid shape");
  if (n == 0) return XLBG_OK;
  if ((unsigned long long)(n + 255) / 256 > 0x7fffffffULL) return fail(XLBG_ERR_ARG, "too many indices");
  int e;
  if ((e = check_ptr(indices, 8, "indices")) || (e = check_ptr(bc_mask, 1, "bc_mask")) ||
      (e = check_ptr(missing_mask, 1, "missing_mask")))
    return e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned g = (unsigned)((n + 255) / 256);
  const int nx = (int)desc->nx, ny = (int)desc->ny, nz = (int)desc->nz;
  const int pad = needs_padding ? 1 : 0;
  if (desc->lattice == XLBG_D2Q9)
    indices_mask<Lattice<0>><<<g, 256, 0, s>>>(indices, n, bc_id, pad, nx, ny, nz, bc_mask, missing_mask);
  else if (desc->lattice == XLBG_D3Q19)
    indices_mask<Lattice<1>><<<g, 256, 0, s>>>(indices, n, bc_id, pad, nx, ny, nz, bc_mask, missing_mask);
  else
    indices_mask<Lattice<2>><<<g, 256, 0, s>>>(indices, n, bc_id, pad, nx, ny, nz, bc_mask, missing_mask);
  const cudaError_t r = cudaGetLastError();
  if (r != cudaSuccess) return fail(XLBG_ERR_CUDA, "indices masker launch: %s", cudaGetErrorString(r));
  return XLBG_OK;
}
