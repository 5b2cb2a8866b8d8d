// Mesh boundary masker: the voxelisation of a triangle mesh into bc_mask /
// missing_mask that XLB's MeshBoundaryMasker performs
// (xlb/operator/boundary_masker/mesh_boundary_masker.py:52-183), as three kernels:
//
//   mesh_precompute: per triangle, its bounds, unit normal and the terms of
//     pre_compute (:64-97);
//   mesh_solid: per (triangle, brick) pair of the caller's list, every voxel of
//     the brick (bricks of B^3 voxels of the grid padded by one cell on every
//     side) whose unit box [low, low + 1] (low = the cell index) the triangle's
//     bounds meet (closed intervals, the BVH query :120) is tested with
//     triangle_box_intersect (:103-117) and set solid on a hit.  Every store
//     writes 1 into a zeroed flag array, so the flags are the OR over all pairs
//     whatever the order.  The projected-edge tests (:110-113) run only with
//     XLBG_MESH_EDGE_TESTS: pre_compute fills its edge matrices by nested
//     subscript stores (m[i][axis0] = ..., :88-95), which in a Warp function
//     write a copy of row i and leave the matrices zero, so by default those
//     tests read 0 >= 0;
//   mesh_mark: from every solid voxel s, id 255 into cell s and, for every
//     l >= 1, the BC id and missing[opp l] into the non-solid cell s - c_l: the
//     marks XLB's kernel gives each cell from its own and its neighbours'
//     voxels (:165-183).
//
// float32 throughout, in the operation order of XLB's functions (the file is
// built with --fmad=false).  The face normal is cross(v1 - v0, v2 - v0) over its
// length; XLB takes Warp's mesh face normal, which may round differently.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xlbg.h"
#include "lattice.cuh"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int check_ptr(const void* p, int align, const char* name);

namespace {

// Per-triangle records in tri_scratch: n_tri base records of kBase floats
// ([0..5] bounds min xyz, max xyz; [6..8] unit normal; [9] dist1; [10] dist2;
// [11] unused), 16-byte aligned and moved as three float4, then n_tri edge
// records of kEdge floats ([0..8] normal_edge0[edge][axis], [9..17]
// normal_edge1, [18..26] dist_edge), written and read with
// XLBG_MESH_EDGE_TESTS only.
constexpr int kBase = 12;
constexpr int kEdge = 27;
static_assert(kBase + kEdge == XLBG_MESH_TRI_FLOATS, "record size");

__device__ __forceinline__ float dot3(const float* a, const float* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

__global__ void mesh_precompute(const float* __restrict__ tri, long long n_tri, int edge_tests, float* __restrict__ rec) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tri) return;
  float v[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) v[i][k] = tri[t * 9 + i * 3 + k];
  float r[kBase];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r[k] = fminf(fminf(v[0][k], v[1][k]), v[2][k]);
    r[3 + k] = fmaxf(fmaxf(v[0][k], v[1][k]), v[2][k]);
  }
  const float e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
  const float e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
  float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
  const float len = sqrtf(dot3(n, n));
#pragma unroll
  for (int k = 0; k < 3; ++k) n[k] = len > 0.0f ? n[k] / len : 0.0f;
  r[6] = n[0];
  r[7] = n[1];
  r[8] = n[2];
  const float corner[3] = {n[0] > 0.0f ? 1.0f : 0.0f, n[1] > 0.0f ? 1.0f : 0.0f, n[2] > 0.0f ? 1.0f : 0.0f};
  const float a[3] = {corner[0] - v[0][0], corner[1] - v[0][1], corner[2] - v[0][2]};
  const float b[3] = {(1.0f - corner[0]) - v[0][0], (1.0f - corner[1]) - v[0][1], (1.0f - corner[2]) - v[0][2]};
  r[9] = dot3(n, a);
  r[10] = dot3(n, b);
  r[11] = 0.0f;
  float4* out = reinterpret_cast<float4*>(rec + t * kBase);
  out[0] = make_float4(r[0], r[1], r[2], r[3]);
  out[1] = make_float4(r[4], r[5], r[6], r[7]);
  out[2] = make_float4(r[8], r[9], r[10], r[11]);
  if (!edge_tests) return;
  float* re = rec + n_tri * kBase + t * kEdge;
  const float ed[3][3] = {{v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]},
                          {v[2][0] - v[1][0], v[2][1] - v[1][1], v[2][2] - v[1][2]},
                          {v[0][0] - v[2][0], v[0][1] - v[2][1], v[0][2] - v[2][2]}};
#pragma unroll
  for (int a0 = 0; a0 < 3; ++a0) {
    const int a2 = (a0 + 2) % 3;
    const float sgn = n[a2] < 0.0f ? -1.0f : 1.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float ne0 = -1.0f * sgn * ed[i][a0];
      const float ne1 = sgn * ed[i][a0];
      re[i * 3 + a0] = ne0;
      re[9 + i * 3 + a0] = ne1;
      re[18 + i * 3 + a0] = -1.0f * (ne0 * v[i][a0] + ne1 * v[i][a0]) + fmaxf(0.0f, ne0) + fmaxf(0.0f, ne1);
    }
  }
}

// Whether the unit box at low meets the triangle of base record r (and, when
// re is not null, passes the projected-edge tests of edge record re).
__device__ __forceinline__ bool box_hits(const float (&low)[3], const float (&r)[kBase], const float* __restrict__ re) {
  bool cand = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) cand = cand && r[k] <= low[k] + 1.0f && r[3 + k] >= low[k];
  if (!cand) return false;
  const float n[3] = {r[6], r[7], r[8]};
  if (!(sqrtf(dot3(n, n)) > 0.0f)) return false;
  const float nl = dot3(n, low);
  if (!((nl + r[9]) * (nl + r[10]) <= 0.0f)) return false;
  if (re == nullptr) return true;
#pragma unroll
  for (int a0 = 0; a0 < 3; ++a0) {
    const int a1 = (a0 + 1) % 3;
#pragma unroll
    for (int i = 0; i < 3; ++i)
      if (!(re[i * 3 + a0] * low[a0] + re[9 + i * 3 + a0] * low[a1] + re[18 + i * 3 + a0] >= 0.0f)) return false;
  }
  return true;
}

__global__ void mesh_solid(const float* __restrict__ rec, long long n_tri, const int32_t* __restrict__ pair_tri,
                           const int32_t* __restrict__ pair_brick, long long n_pairs, int brick, int nbx, int nby,
                           int nbz, int px, int py, int pz, int edge_tests, uint8_t* __restrict__ solid) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_pairs) return;
  const int t = pair_tri[q];
  const int b = pair_brick[q];
  if (t < 0 || t >= n_tri || b < 0 || (long long)b >= (long long)nbx * nby * nbz) return;  // skipped
  float r[kBase];
  const float4* in = reinterpret_cast<const float4*>(rec + (long long)t * kBase);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 x = in[k];
    r[4 * k] = x.x;
    r[4 * k + 1] = x.y;
    r[4 * k + 2] = x.z;
    r[4 * k + 3] = x.w;
  }
  const float* re = edge_tests ? rec + n_tri * kBase + (long long)t * kEdge : nullptr;
  const int bo[3] = {(b / (nby * nbz)) * brick, ((b / nbz) % nby) * brick, (b % nbz) * brick};
  const int pd[3] = {px, py, pz};
  int p0[3], p1[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // voxel p has box [p - 1, p]: the bounds [lo, hi] meet it iff ceil(lo) <= p <= floor(hi) + 1.
    // Clamped to the brick in float before converting, so coordinates far outside
    // the grid (or not finite: every comparison with NaN is false) cannot overflow.
    const float lo = ceilf(r[k]), hi = floorf(r[3 + k]) + 1.0f;
    const float lim0 = (float)bo[k], lim1 = (float)min(bo[k] + brick - 1, pd[k] - 1);
    if (!(lo <= lim1 && hi >= lim0)) return;  // the bounds miss this brick
    p0[k] = (int)fmaxf(lo, lim0);
    p1[k] = (int)fminf(hi, lim1);
  }
  for (int i = p0[0]; i <= p1[0]; ++i)
    for (int j = p0[1]; j <= p1[1]; ++j)
      for (int k = p0[2]; k <= p1[2]; ++k) {
        const long long p = ((long long)i * py + j) * pz + k;
        if (solid[p]) continue;
        const float low[3] = {(float)(i - 1), (float)(j - 1), (float)(k - 1)};
        if (box_hits(low, r, re)) solid[p] = 1;
      }
}

// One thread per voxel of the padded grid.  For each solid voxel s: the cell s
// (if in the domain) gets 255; for every l >= 1 the cell x = s - c_l, if in the
// domain and not solid, gets bc_id and missing[opp l] (its neighbour x + c_l is
// s).  Every store writes the one value its address can receive (255 only into
// solid cells, bc_id and 1 only into non-solid ones), so the result does not
// depend on the order of the threads.
template <class L>
__global__ void mesh_mark(const uint8_t* __restrict__ solid, long long np, int nx, int ny, int nz, int bc_id,
                          uint8_t* __restrict__ bc_mask, uint8_t* __restrict__ missing) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np || !solid[p]) return;
  const int py = ny + 2, pz = nz + 2;
  const long long n = (long long)nx * ny * nz;
  const int si = (int)(p / ((long long)py * pz)) - 1;
  const int sj = (int)((p / pz) % py) - 1;
  const int sk = (int)(p % pz) - 1;
  if (si >= 0 && si < nx && sj >= 0 && sj < ny && sk >= 0 && sk < nz) bc_mask[((long long)si * ny + sj) * nz + sk] = 255;
#pragma unroll
  for (int l = 1; l < L::Q; ++l) {
    const int xi = si - L::c(l, 0), xj = sj - L::c(l, 1), xk = sk - L::c(l, 2);
    if (xi < 0 || xi >= nx || xj < 0 || xj >= ny || xk < 0 || xk >= nz) continue;
    if (solid[((long long)(xi + 1) * py + (xj + 1)) * pz + (xk + 1)]) continue;
    const long long cell = ((long long)xi * ny + xj) * nz + xk;
    bc_mask[cell] = (uint8_t)bc_id;
    missing[(long long)opp<L>(l) * n + cell] = 1;
  }
}

}  // namespace
}  // namespace xlbg

using namespace xlbg;

extern "C" int xlbg_mesh_mask(const xlbg_desc* desc, const float* tri, int64_t n_tri, const int32_t* pair_tri,
                              const int32_t* pair_brick, int64_t n_pairs, int32_t brick, int32_t bc_id, int32_t flags,
                              float* tri_scratch, uint8_t* solid_scratch, uint8_t* bc_mask, uint8_t* missing_mask,
                              void* stream) {
  if (!desc || desc->abi_version != XLBG_ABI_VERSION) return fail(XLBG_ERR_ARG, "bad descriptor");
  if (desc->lattice == XLBG_D2Q9) return fail(XLBG_ERR_UNSUPPORTED, "the mesh masker is 3D only");
  if (desc->lattice != XLBG_D3Q19 && desc->lattice != XLBG_D3Q27) return fail(XLBG_ERR_ARG, "bad lattice");
  if (n_tri < 0 || n_tri >= (1LL << 31) || n_pairs < 0 || n_pairs >= (1LL << 38) || brick < 1 || brick > 1024 ||
      bc_id < 1 || bc_id > 254)
    return fail(XLBG_ERR_ARG, "bad n_tri, n_pairs, brick or bc_id");
  if (flags & ~XLBG_MESH_EDGE_TESTS) return fail(XLBG_ERR_ARG, "unknown mesh masker flags %d", flags);
  // padded cell indices and coordinates stay exact in int and float32; the
  // one-voxel-per-thread grids stay below 2^31 blocks of 256
  if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1 || desc->nx > (1 << 22) || desc->ny > (1 << 22) ||
      desc->nz > (1 << 22) || (desc->nx + 2) * (desc->ny + 2) * (desc->nz + 2) >= (1LL << 38))
    return fail(XLBG_ERR_ARG, "bad grid shape");
  const long long nb = (long long)((desc->nx + 2 + brick - 1) / brick) * ((desc->ny + 2 + brick - 1) / brick) *
                       ((desc->nz + 2 + brick - 1) / brick);
  if (nb >= (1LL << 31) - 1) return fail(XLBG_ERR_ARG, "too many bricks (%lld); use a larger brick", nb);
  int e;
  if ((e = check_ptr(solid_scratch, 16, "solid_scratch")) || (e = check_ptr(bc_mask, 1, "bc_mask")) ||
      (e = check_ptr(missing_mask, 1, "missing_mask")))
    return e;
  if (n_tri > 0 && ((e = check_ptr(tri, 4, "tri")) || (e = check_ptr(tri_scratch, 16, "tri_scratch")))) return e;
  if (n_pairs > 0 && ((e = check_ptr(pair_tri, 4, "pair_tri")) || (e = check_ptr(pair_brick, 4, "pair_brick"))))
    return e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nx = (int)desc->nx, ny = (int)desc->ny, nz = (int)desc->nz;
  const int px = nx + 2, py = ny + 2, pz = nz + 2;
  const int nbx = (px + brick - 1) / brick, nby = (py + brick - 1) / brick, nbz = (pz + brick - 1) / brick;
  const int et = (flags & XLBG_MESH_EDGE_TESTS) ? 1 : 0;
  const long long np = (long long)px * py * pz;
  const long long n_words = (np + 15) / 16;
  cudaError_t r = cudaMemsetAsync(solid_scratch, 0, (size_t)n_words * 16, s);
  if (r != cudaSuccess) return fail(XLBG_ERR_CUDA, "mesh masker memset: %s", cudaGetErrorString(r));
  if (n_tri > 0 && n_pairs > 0) {
    mesh_precompute<<<(unsigned)((n_tri + 255) / 256), 256, 0, s>>>(tri, n_tri, et, tri_scratch);
    mesh_solid<<<(unsigned)((n_pairs + 255) / 256), 256, 0, s>>>(tri_scratch, n_tri, pair_tri, pair_brick, n_pairs,
                                                                 brick, nbx, nby, nbz, px, py, pz, et, solid_scratch);
  }
  const unsigned g = (unsigned)((np + 255) / 256);
  if (desc->lattice == XLBG_D3Q19)
    mesh_mark<Lattice<1>><<<g, 256, 0, s>>>(solid_scratch, np, nx, ny, nz, bc_id, bc_mask, missing_mask);
  else
    mesh_mark<Lattice<2>><<<g, 256, 0, s>>>(solid_scratch, np, nx, ny, nz, bc_id, bc_mask, missing_mask);
  r = cudaGetLastError();
  if (r != cudaSuccess) return fail(XLBG_ERR_CUDA, "mesh masker launch: %s", cudaGetErrorString(r));
  return XLBG_OK;
}
