"""CPU restatement of XLB's mesh boundary masker -- TEST INFRASTRUCTURE ONLY.

Follows xlb/operator/boundary_masker/mesh_boundary_masker.py:52-183, in float32
with the operation order written there, over every (voxel, triangle) pair (no
acceleration structure, so small grids only):

* voxel (i, j, k) is the unit box [low, low + 1] with low = (i, j, k)
  (cell centre minus one half, :54-60, :172-176);
* candidate triangles are those whose axis-aligned bounds overlap that box,
  closed intervals (what the mesh BVH query :120 returns);
* per triangle the terms of ``pre_compute`` (:64-97) from its vertices and unit
  normal, and the test of ``triangle_box_intersect`` (:103-117);
* ``pre_compute`` fills its three edge matrices with nested subscript stores
  (``m[i][axis0] = ...``, :88-95).  In a Warp function ``m[i]`` of a local matrix
  is a copy of row i, so those stores leave the matrices zero and every
  projected-edge test of :110-113 reads ``0 >= 0``: a voxel is solid when a
  candidate triangle's plane separates two opposite corners of the voxel.  That
  is the default here (``edge_tests=False``).  ``edge_tests=True`` applies the
  stores as written (normal_edge0 = -sgn*e[axis0], normal_edge1 = sgn*e[axis0],
  dist_edge from vertex axis0 twice), for a Warp that gives ``m[i][j] = x``
  element-store semantics;
* a voxel that intersects the mesh gets id 255; every other voxel with an
  intersecting neighbour x + c_l (l >= 1) gets the BC id and missing[opp l]
  (:165-183).

The face normal is cross(v1 - v0, v2 - v0) divided by its length (sqrt of the
dot product), each operation correctly rounded in float32; XLB takes Warp's
mesh face normal, whose rounding may differ in the last bit.

Only ``tests/`` may import this module.
"""

import numpy as np

F = np.float32


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def face_normals(tri):
    """tri (T, 3, 3) float32 vertices -> (T, 3) unit normals (zero for degenerate faces)."""
    e1 = tri[:, 1] - tri[:, 0]
    e2 = tri[:, 2] - tri[:, 0]
    n = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                  e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1).astype(F)
    length = np.sqrt(_dot(n, n)).astype(F)
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where(length[:, None] > 0, n / length[:, None], F(0)).astype(F)
    return out


def pre_compute(tri, normal):
    """mesh_boundary_masker.py:64-97 for every triangle: dist1, dist2 (T,), and
    normal_edge0, normal_edge1, dist_edge (T, 3 edges, 3 axes)."""
    v = tri
    corner = (normal > 0).astype(F)
    dist1 = _dot(normal, corner - v[:, 0]).astype(F)
    dist2 = _dot(normal, (F(1) - corner) - v[:, 0]).astype(F)
    edges = np.stack([v[:, 1] - v[:, 0], v[:, 2] - v[:, 1], v[:, 0] - v[:, 2]], axis=1).astype(F)  # (T, edge, axis)
    ne0 = np.zeros_like(edges)
    ne1 = np.zeros_like(edges)
    de = np.zeros_like(edges)
    for a0 in range(3):
        a2 = (a0 + 2) % 3
        sgn = np.where(normal[:, a2] < 0, F(-1), F(1)).astype(F)
        for i in range(3):
            ne0[:, i, a0] = F(-1) * sgn * edges[:, i, a0]
            ne1[:, i, a0] = sgn * edges[:, i, a0]
            de[:, i, a0] = (F(-1) * (ne0[:, i, a0] * v[:, i, a0] + ne1[:, i, a0] * v[:, i, a0])
                            + np.maximum(F(0), ne0[:, i, a0]) + np.maximum(F(0), ne1[:, i, a0]))
    return dist1, dist2, ne0, ne1, de


def voxel_solid(low, tri, pre, normal, edge_tests=False):
    """Whether the unit voxels at low (N, 3) intersect the mesh: (N,) bool."""
    dist1, dist2, ne0, ne1, de = pre
    tmin = tri.min(axis=1)
    tmax = tri.max(axis=1)
    lo = low[:, None, :]
    hi = (low + F(1))[:, None, :]
    cand = np.all((tmin[None] <= hi) & (tmax[None] >= lo), axis=2)  # (N, T)
    nlen = np.sqrt(_dot(normal, normal))
    nl = _dot(normal[None], lo)  # (N, T)
    plane = (nlen[None] > 0) & ((nl + dist1[None]) * (nl + dist2[None]) <= 0)
    hit = plane.copy()
    for a0 in range(3 if edge_tests else 0):
        a1 = (a0 + 1) % 3
        for i in range(3):
            t = ne0[None, :, i, a0] * low[:, None, a0] + ne1[None, :, i, a0] * low[:, None, a1] + de[None, :, i, a0]
            hit &= t >= 0
    return np.any(cand & hit, axis=1)


def mask(lat, shape, tri, bc_id, bc_mask, missing, edge_tests=False):
    """Apply the mesh masker for one BC in place to (bc_mask, missing) numpy
    arrays of XLB's shapes (1, nx, ny, nz) and (Q, nx, ny, nz); returns them.
    tri is (T, 3, 3): vertex v of triangle t at tri[t, v]."""
    tri = np.asarray(tri, dtype=F)
    normal = face_normals(tri)
    pre = pre_compute(tri, normal)
    nx, ny, nz = shape
    # solid flags on the grid padded by one cell on every side
    g = np.stack(np.meshgrid(np.arange(-1, nx + 1), np.arange(-1, ny + 1), np.arange(-1, nz + 1), indexing="ij"),
                 axis=-1).reshape(-1, 3).astype(F)
    solid = voxel_solid(g, tri, pre, normal, edge_tests).reshape(nx + 2, ny + 2, nz + 2)
    inner = solid[1:-1, 1:-1, 1:-1]
    for l in range(1, lat.q):
        cx, cy, cz = (int(lat.c[d, l]) for d in range(3))
        nb = solid[1 + cx:1 + cx + nx, 1 + cy:1 + cy + ny, 1 + cz:1 + cz + nz]
        sel = (~inner) & nb
        bc_mask[0][sel] = bc_id
        missing[lat.opp[l]][sel] = True
    bc_mask[0][inner] = 255
    return bc_mask, missing
