"""CPU restatement of XLB's ray-traced mesh renderer -- TEST INFRASTRUCTURE ONLY.

Follows examples/out_of_core/operators/mesh_renderer.py:81-187 (``_render_mesh``)
in float32, vectorised over pixels, brute force over triangles (small scenes):

* ray per pixel: NDC from the pixel index (:103-106), camera basis of
  ``create_view_matrix`` (:34-49), direction normalize((sx, sy, -1)) rotated
  into world space and normalised again (:112-123);
* closest hit with t < depth_buffer[i, j] (the query's max_t, :126-128);
* colour: vertex colours weighted by the hit's barycentrics u (vertex 0), v
  (vertex 1) and 1 - u - v (vertex 2) (:136-152), ``normal_based_shading``
  (:51-78), gamma pow(clamp(c, 0, 1), 1 / gamma) (:163-168); RGBA and depth
  written on a hit only (:170-175).

The ray-triangle test is Warp's ``mesh_query_ray``, which is not part of the XLB
tree; it is restated here from the published watertight algorithm (Woop,
Benthin and Wald, "Watertight Ray/Triangle Intersection", JCGT 2013) without its
double-precision fallback: shear to the ray's dominant axis, edge functions U,
V, W, reject mixed signs and det = 0, t = T / det; u = U / det weights vertex 0,
v = V / det vertex 1.  The hit normal is normalize(cross(v1 - v0, v2 - v0)).  A
hit needs t >= 0.  Among hits with equal t the lowest face index wins (Warp's
choice depends on its BVH order).  The camera and shading code is pinned to
XLB's source by tests/golden/make_golden_render.py; the intersection is not
(parity of that part unpinned against Warp).

Only ``tests/`` may import this module.
"""

import math

import numpy as np

F = np.float32


def _norm(v):
    """v (..., 3) / length, float32, zero where the length is zero."""
    n = np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(n[..., None] > 0, v / n[..., None], F(0)).astype(F)


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1).astype(F)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def rays(width, height, camera_pos, camera_target, camera_up, fov_degrees):
    """(H, W, 3) float32 world-space ray directions (mesh_renderer.py:98-123)."""
    eye, target, up = (np.asarray(v, dtype=F) for v in (camera_pos, camera_target, camera_up))
    forward = _norm(target - eye)
    right = _norm(_cross(forward, up))
    up2 = _norm(_cross(right, forward))
    # view[r, c]: columns right, up, -forward (the rotation part of the view matrix)
    view = np.stack([right, up2, -forward], axis=1).astype(F)
    aspect = F(width) / F(height)
    fov = F(fov_degrees) * F(math.pi / 180.0)
    tan_fov = F(math.tan(float(fov * F(0.5))))
    j = np.arange(width, dtype=F)[None, :]
    i = np.arange(height, dtype=F)[:, None]
    sx = (F(2) * j / F(width) - F(1)) * aspect * tan_fov
    sy = (F(1) - F(2) * i / F(height)) * tan_fov
    sx, sy = np.broadcast_arrays(sx, sy)
    d = _norm(np.stack([sx, sy, np.full_like(sx, -1.0)], axis=-1).astype(F))
    rd = np.stack([(d[..., 0] * view[r, 0] + d[..., 1] * view[r, 1]) + d[..., 2] * view[r, 2] for r in range(3)],
                  axis=-1).astype(F)
    return _norm(rd)


def woop(org, d, p0, p1, p2):
    """Watertight ray-triangle test for rays d (P, 3) from org (3,) against one
    triangle: (hit (P,) bool, t, u, v) float32."""
    ad = np.abs(d)
    kz = np.argmax(ad, axis=1)  # first of equal maxima
    kx = (kz + 1) % 3
    ky = (kx + 1) % 3
    neg = np.take_along_axis(d, kz[:, None], 1)[:, 0] < 0
    kx, ky = np.where(neg, ky, kx), np.where(neg, kx, ky)
    g = lambda v, k: np.take_along_axis(v, k[:, None], 1)[:, 0] if v.ndim == 2 else v[k]  # noqa: E731
    dz = g(d, kz)
    sx = g(d, kx) / dz
    sy = g(d, ky) / dz
    sz = F(1) / dz
    a, b, c = (np.asarray(p, dtype=F) - org for p in (p0, p1, p2))
    ax = g(a, kx) - sx * g(a, kz)
    ay = g(a, ky) - sy * g(a, kz)
    bx = g(b, kx) - sx * g(b, kz)
    by = g(b, ky) - sy * g(b, kz)
    cx = g(c, kx) - sx * g(c, kz)
    cy = g(c, ky) - sy * g(c, kz)
    U = cx * by - cy * bx
    V = ax * cy - ay * cx
    W = bx * ay - by * ax
    mixed = ((U < 0) | (V < 0) | (W < 0)) & ((U > 0) | (V > 0) | (W > 0))
    det = (U + V) + W
    T = ((U * (sz * g(a, kz)) + V * (sz * g(b, kz))) + W * (sz * g(c, kz)))
    with np.errstate(invalid="ignore", divide="ignore"):
        rcp = F(1) / det
    hit = ~mixed & (det != 0)
    t = (T * rcp).astype(F)
    u = (U * rcp).astype(F)
    v = (V * rcp).astype(F)
    return hit & (t >= 0), t, u, v


def render(points, indices, vertex_colors, pixel_buffer, depth_buffer, camera_pos=(0.0, 1.0, 2.0),
           camera_target=(0.0, 0.0, 0.0), camera_up=(0.0, 1.0, 0.0), fov_degrees=60.0, ambient_intensity=0.05,
           edge_sharpness=1.0, gamma=1.0):
    """Render in place into pixel_buffer (H, W, 4) and depth_buffer (H, W), float32
    numpy arrays; returns (pixel_buffer, depth_buffer, face (H, W) int, -1 = miss)."""
    pts = np.asarray(points, dtype=F)
    ind = np.asarray(indices, dtype=np.int64).reshape(-1, 3)
    col = np.asarray(vertex_colors, dtype=F)
    h, w = depth_buffer.shape
    rd = rays(w, h, camera_pos, camera_target, camera_up, fov_degrees).reshape(-1, 3)
    org = np.asarray(camera_pos, dtype=F)
    best_t = depth_buffer.reshape(-1).astype(F).copy()
    best_f = np.full(best_t.shape, -1, dtype=np.int64)
    best_u = np.zeros_like(best_t)
    best_v = np.zeros_like(best_t)
    for f, (i0, i1, i2) in enumerate(ind):
        hit, t, u, v = woop(org, rd, pts[i0], pts[i1], pts[i2])
        take = hit & (t < best_t)  # strict: the lower face index keeps an equal t
        best_t = np.where(take, t, best_t)
        best_f = np.where(take, f, best_f)
        best_u = np.where(take, u, best_u)
        best_v = np.where(take, v, best_v)
    sel = best_f >= 0
    if sel.any():
        fi = ind[best_f[sel]]
        p0, p1, p2 = pts[fi[:, 0]], pts[fi[:, 1]], pts[fi[:, 2]]
        n = _norm(_norm(_cross(p1 - p0, p2 - p0)))  # the query's unit normal, normalised again (:132)
        u, v = best_u[sel], best_v[sel]
        w2 = (F(1) - u) - v
        base = ((col[fi[:, 0]] * u[:, None] + col[fi[:, 1]] * v[:, None]) + col[fi[:, 2]] * w2[:, None]).astype(F)
        vv = _norm(rd[sel])
        nn = _norm(n)
        ndv = _dot(nn, vv)
        ndv = np.where(ndv < 0, -ndv, ndv).astype(F)
        with np.errstate(invalid="ignore", divide="ignore"):
            diffuse = np.power(ndv, F(edge_sharpness)).astype(F)
        light = (F(ambient_intensity) + diffuse).astype(F)
        color = (base * light[:, None]).astype(F)
        with np.errstate(invalid="ignore", divide="ignore"):
            color = np.power(np.clip(color, F(0), F(1)), F(1) / F(gamma)).astype(F)
        pb = pixel_buffer.reshape(-1, 4)
        pb[sel, 0:3] = color
        pb[sel, 3] = F(1)
        depth_buffer.reshape(-1)[sel] = best_t[sel]
    return pixel_buffer, depth_buffer, best_f.reshape(h, w)
