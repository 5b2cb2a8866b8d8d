// Ray-traced mesh renderer: the per-pixel work of the MeshRenderer operator in
// XLB's out-of-core example (examples/out_of_core/operators/mesh_renderer.py:81-187).
//
// One thread per pixel.  The ray is built as XLB builds it (NDC :103-106, the
// view basis of create_view_matrix :34-49, normalize((sx, sy, -1)) rotated into
// world space and normalised :112-123), in float32 with XLB's operation order
// (the file is built with --fmad=false).  The closest hit with t < depth[i, j]
// comes from a walk through a uniform grid of triangle lists (3D DDA,
// Amanatides and Woo): every triangle listed in a visited cell is tested with
// the watertight ray-triangle test (Woop, Benthin and Wald, JCGT 2013, without
// its double-precision fallback) and the lowest (t, face) is kept, so the
// result does not depend on the visiting order; the walk stops once the next
// cell starts beyond the best hit.  XLB gets the hit from Warp's mesh BVH
// query, whose tie order between equal t is its traversal order.  Colour,
// shading and gamma follow :130-175.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xlbg.h"

namespace xlbg {

int fail(int code, const char* fmt, ...);
int check_ptr(const void* p, int align, const char* name);

namespace {

struct v3 {
  float x, y, z;
};
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ v3 normalize(v3 a) {
  const float n = sqrtf(dot(a, a));
  if (n > 0.0f) return {a.x / n, a.y / n, a.z / n};
  return {0.0f, 0.0f, 0.0f};
}
__device__ __forceinline__ float comp(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ v3 load3(const float* p, long long i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

// Watertight test of the ray (org, d) against triangle (p0, p1, p2), with the
// ray's shear precomputed: kx, ky, kz and S = (d[kx] / d[kz], d[ky] / d[kz], 1 / d[kz]).
__device__ __forceinline__ bool woop(v3 org, int kx, int ky, int kz, float sx, float sy, float sz, v3 p0, v3 p1,
                                     v3 p2, float& t, float& u, float& v) {
  const v3 a = sub(p0, org), b = sub(p1, org), c = sub(p2, org);
  const float ax = comp(a, kx) - sx * comp(a, kz), ay = comp(a, ky) - sy * comp(a, kz);
  const float bx = comp(b, kx) - sx * comp(b, kz), by = comp(b, ky) - sy * comp(b, kz);
  const float cx = comp(c, kx) - sx * comp(c, kz), cy = comp(c, ky) - sy * comp(c, kz);
  const float U = cx * by - cy * bx;
  const float V = ax * cy - ay * cx;
  const float W = bx * ay - by * ax;
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = (U + V) + W;
  if (det == 0.0f) return false;
  const float T = (U * (sz * comp(a, kz)) + V * (sz * comp(b, kz))) + W * (sz * comp(c, kz));
  const float rcp = 1.0f / det;
  t = T * rcp;
  if (!(t >= 0.0f)) return false;
  u = U * rcp;
  v = V * rcp;
  return true;
}

struct Cam {
  v3 eye, target, up;
  float fov_degrees, ambient, sharpness, gamma;
};

struct Grid {
  v3 lo, cell;
  int nx, ny, nz;
  const int32_t* start;
  const int32_t* tris;
};

__global__ void render_kernel(const float* __restrict__ pts, long long n_points, const int32_t* __restrict__ ind,
                              long long n_tri,
                              const float* __restrict__ colors, const Grid g, const Cam cam, int height, int width,
                              float* __restrict__ pixel, float* __restrict__ depth, int32_t* __restrict__ face_out,
                              int* __restrict__ err) {
  // a block covers 16 x 8 pixels, each warp an 8 x 4 tile (neighbouring rays walk
  // neighbouring cells, so the warp's lanes stay together longer)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  const int j = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  if (i >= height || j >= width) return;
  const long long pix = (long long)i * width + j;
  // ---- the ray (mesh_renderer.py:98-123) ----
  const float aspect = (float)width / (float)height;
  const float fov = cam.fov_degrees * 0.017453292519943295f;
  const float tan_fov = tanf(fov * 0.5f);
  const float sx = (2.0f * (float)j / (float)width - 1.0f) * aspect * tan_fov;
  const float sy = (1.0f - 2.0f * (float)i / (float)height) * tan_fov;
  const v3 forward = normalize(sub(cam.target, cam.eye));
  const v3 right = normalize(cross(forward, cam.up));
  const v3 up = normalize(cross(right, forward));
  const v3 d = normalize(v3{sx, sy, -1.0f});
  const v3 rd = normalize(v3{(d.x * right.x + d.y * up.x) + d.z * -forward.x,
                             (d.x * right.y + d.y * up.y) + d.z * -forward.y,
                             (d.x * right.z + d.y * up.z) + d.z * -forward.z});
  const v3 org = cam.eye;
  // ---- shear of the watertight test ----
  int kz = 0;
  if (fabsf(rd.y) > fabsf(rd.x)) kz = 1;
  if (fabsf(rd.z) > fabsf(comp(rd, kz))) kz = 2;
  int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
  if (comp(rd, kz) < 0.0f) {
    const int s = kx;
    kx = ky;
    ky = s;
  }
  const float dz = comp(rd, kz);
  const float shx = comp(rd, kx) / dz, shy = comp(rd, ky) / dz, shz = 1.0f / dz;
  // ---- walk the grid ----
  float best_t = depth[pix];
  int best_f = -1;
  float best_u = 0.0f, best_v = 0.0f;
  const float dir[3] = {rd.x, rd.y, rd.z}, o[3] = {org.x, org.y, org.z};
  const float lo[3] = {g.lo.x, g.lo.y, g.lo.z}, cs[3] = {g.cell.x, g.cell.y, g.cell.z};
  const int dims[3] = {g.nx, g.ny, g.nz};
  float t0 = 0.0f, t1 = INFINITY;
  bool inside = true;
  for (int k = 0; k < 3; ++k) {
    const float hi = lo[k] + cs[k] * (float)dims[k];
    if (dir[k] == 0.0f) {
      if (o[k] < lo[k] || o[k] > hi) inside = false;
    } else {
      float ta = (lo[k] - o[k]) / dir[k], tb = (hi - o[k]) / dir[k];
      if (ta > tb) {
        const float s = ta;
        ta = tb;
        tb = s;
      }
      t0 = fmaxf(t0, ta);
      t1 = fminf(t1, tb);
    }
  }
  if (inside && t0 <= t1 && t0 < best_t) {
    int c[3], step[3];
    float tmax[3], tdelta[3];
    for (int k = 0; k < 3; ++k) {
      const float p = o[k] + t0 * dir[k];
      int ck = (int)floorf((p - lo[k]) / cs[k]);
      c[k] = ck < 0 ? 0 : (ck >= dims[k] ? dims[k] - 1 : ck);
      if (dir[k] > 0.0f) {
        step[k] = 1;
        tmax[k] = (lo[k] + cs[k] * (float)(c[k] + 1) - o[k]) / dir[k];
        tdelta[k] = cs[k] / dir[k];
      } else if (dir[k] < 0.0f) {
        step[k] = -1;
        tmax[k] = (lo[k] + cs[k] * (float)c[k] - o[k]) / dir[k];
        tdelta[k] = -cs[k] / dir[k];
      } else {
        step[k] = 0;
        tmax[k] = INFINITY;
        tdelta[k] = INFINITY;
      }
    }
    const long long max_cells = (long long)dims[0] + dims[1] + dims[2] + 3;  // a line crosses at most this many
    for (long long visited = 0; visited < max_cells; ++visited) {
      const long long cell = ((long long)c[0] * dims[1] + c[1]) * dims[2] + c[2];
      for (int q = g.start[cell]; q < g.start[cell + 1]; ++q) {
        const int f = g.tris[q];
        const long long a0 = (f >= 0 && f < n_tri) ? ind[3LL * f] : -1;
        const long long a1 = (f >= 0 && f < n_tri) ? ind[3LL * f + 1] : -1;
        const long long a2 = (f >= 0 && f < n_tri) ? ind[3LL * f + 2] : -1;
        if (a0 < 0 || a0 >= n_points || a1 < 0 || a1 >= n_points || a2 < 0 || a2 >= n_points) {
          atomicAdd(err, 1);  // a malformed list or index: report, skip the entry
          continue;
        }
        float t, u, v;
        if (woop(org, kx, ky, kz, shx, shy, shz, load3(pts, a0), load3(pts, a1), load3(pts, a2), t, u, v) &&
            (t < best_t || (t == best_t && best_f >= 0 && f < best_f))) {
          best_t = t;
          best_f = f;
          best_u = u;
          best_v = v;
        }
      }
      // leave through the nearest cell face; stop once the next cell starts
      // beyond the best hit (with a margin for the rounding of the walk)
      int k = 0;
      if (tmax[1] < tmax[k]) k = 1;
      if (tmax[2] < tmax[k]) k = 2;
      const float t_exit = tmax[k];
      if (best_f >= 0 && t_exit > best_t * 1.0001f + 1e-6f) break;
      if (t_exit >= depth[pix] * 1.0001f + 1e-6f) break;
      c[k] += step[k];
      if (c[k] < 0 || c[k] >= dims[k]) break;
      tmax[k] += tdelta[k];
    }
  }
  if (face_out) face_out[pix] = best_f;
  if (best_f < 0) return;
  // ---- colour and shading (mesh_renderer.py:130-175) ----
  const long long i0 = ind[3LL * best_f], i1 = ind[3LL * best_f + 1], i2 = ind[3LL * best_f + 2];
  const v3 p0 = load3(pts, i0), p1 = load3(pts, i1), p2 = load3(pts, i2);
  const v3 n = normalize(normalize(cross(sub(p1, p0), sub(p2, p0))));
  const float w0 = best_u, w1 = best_v, w2 = (1.0f - best_u) - best_v;
  const v3 c0 = load3(colors, i0), c1 = load3(colors, i1), c2 = load3(colors, i2);
  const v3 base = {(c0.x * w0 + c1.x * w1) + c2.x * w2, (c0.y * w0 + c1.y * w1) + c2.y * w2,
                   (c0.z * w0 + c1.z * w1) + c2.z * w2};
  const v3 nn = normalize(n), vv = normalize(rd);
  float ndv = dot(nn, vv);
  if (ndv < 0.0f) ndv = -ndv;
  const float light = cam.ambient + powf(ndv, cam.sharpness);
  const float inv_gamma = 1.0f / cam.gamma;
  const float rgb[3] = {base.x * light, base.y * light, base.z * light};
  float* out = pixel + 4 * pix;
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = powf(fminf(fmaxf(rgb[k], 0.0f), 1.0f), inv_gamma);
  out[3] = 1.0f;
  depth[pix] = best_t;
}

}  // namespace
}  // namespace xlbg

using namespace xlbg;

extern "C" int xlbg_render_mesh(const float* points, int64_t n_points, const int32_t* indices, int64_t n_tri,
                                const float* vertex_colors, const xlbg_tri_grid* grid, const xlbg_camera* camera,
                                int32_t height, int32_t width, float* pixel, float* depth, int32_t* face_out,
                                int32_t* err_count, void* stream) {
  if (!grid || !camera) return fail(XLBG_ERR_ARG, "grid or camera is NULL");
  if (n_points < 0 || n_tri < 0 || n_tri >= (1LL << 31) || height < 1 || width < 1 || height > 65535 * 8)
    return fail(XLBG_ERR_ARG, "bad sizes");
  if (grid->dims[0] < 1 || grid->dims[1] < 1 || grid->dims[2] < 1 ||
      (long long)grid->dims[0] * grid->dims[1] * grid->dims[2] >= (1LL << 31) - 1)
    return fail(XLBG_ERR_ARG, "bad grid dims");
  if (!(grid->cell[0] > 0.0f && grid->cell[1] > 0.0f && grid->cell[2] > 0.0f))
    return fail(XLBG_ERR_ARG, "grid cells must have positive size");
  int e;
  if ((e = check_ptr(pixel, 4, "pixel")) || (e = check_ptr(depth, 4, "depth")) ||
      (e = check_ptr(grid->cell_start, 4, "cell_start")) || (e = check_ptr(err_count, 4, "err_count")))
    return e;
  if (n_tri > 0 && ((e = check_ptr(points, 4, "points")) || (e = check_ptr(indices, 4, "indices")) ||
                    (e = check_ptr(vertex_colors, 4, "vertex_colors")) || (e = check_ptr(grid->cell_tris, 4, "cell_tris"))))
    return e;
  Grid g;
  g.lo = {grid->lo[0], grid->lo[1], grid->lo[2]};
  g.cell = {grid->cell[0], grid->cell[1], grid->cell[2]};
  g.nx = grid->dims[0];
  g.ny = grid->dims[1];
  g.nz = grid->dims[2];
  g.start = grid->cell_start;
  g.tris = grid->cell_tris;
  Cam c;
  c.eye = {camera->eye[0], camera->eye[1], camera->eye[2]};
  c.target = {camera->target[0], camera->target[1], camera->target[2]};
  c.up = {camera->up[0], camera->up[1], camera->up[2]};
  c.fov_degrees = camera->fov_degrees;
  c.ambient = camera->ambient_intensity;
  c.sharpness = camera->edge_sharpness;
  c.gamma = camera->gamma;
  const dim3 blocks((unsigned)((width + 15) / 16), (unsigned)((height + 7) / 8));
  render_kernel<<<blocks, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      points, n_points, indices, n_tri, vertex_colors, g, c, height, width, pixel, depth, face_out, err_count);
  const cudaError_t r = cudaGetLastError();
  if (r != cudaSuccess) return fail(XLBG_ERR_CUDA, "render launch: %s", cudaGetErrorString(r));
  return XLBG_OK;
}
