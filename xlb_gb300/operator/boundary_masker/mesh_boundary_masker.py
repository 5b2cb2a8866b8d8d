"""bc_mask / missing_mask from a triangle mesh (set-up, not timed).

Follows XLB's MeshBoundaryMasker (xlb/operator/boundary_masker/mesh_boundary_masker.py):
the same checks and messages (:191-212), the same voxel test and marking
(:52-183), computed by the CUDA kernels of ``xlbg_mesh_mask``.  XLB builds a
Warp mesh with a BVH and, per cell, queries it for the cell's voxel and its
Q - 1 neighbours' voxels; here every voxel of the grid padded by one cell is
tested once (solid flags): one thread per (triangle, brick of ``brick``^3
voxels) pair tests the voxels of the brick that the triangle's bounds meet,
and a second kernel marks the cells from the flags.

The vertices are a triangle soup, (N, 3) with consecutive triples forming a
triangle (XLB's mesh indices are ``arange(N)``), in grid units, converted to
float32 as ``wp.array(..., dtype=wp.vec3)`` does.

``edge_tests``: XLB's ``pre_compute`` fills its edge matrices with nested
subscript stores (``m[i][axis0] = ...``), which in a Warp function write a copy
of row i and leave the matrices zero; its projected-edge tests then always
pass, and a voxel is solid when a triangle's bounds meet it and the triangle's
plane separates two opposite corners of it.  That is the default.
``edge_tests=True`` evaluates those tests with the terms the stores compute.
"""

import numpy as np
import torch

from xlb_gb300 import _lib
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc


def brick_pairs(tri, shape, brick):
    """Work list of the solid-flag kernel: every (triangle, brick) pair where
    the triangle's bounds meet a voxel of the brick.

    tri: (T, 3, 3) float32 tensor (any device); shape: (nx, ny, nz).  Voxel p of
    the padded grid (p = cell index + 1 per axis) is the box [p - 1, p]; a
    triangle's bounds [lo, hi] meet it iff lo <= p and hi >= p - 1, i.e. p in
    [ceil(lo), floor(hi) + 1].  Returns (pair_tri, pair_brick) int32 tensors on
    tri's device, bricks numbered (bx * nby + by) * nbz + bz: first the
    triangles that lie in one brick, then the pairs of the others, grouped by
    triangle.
    """
    dev = tri.device
    pdim = torch.tensor([s + 2 for s in shape], dtype=torch.int64, device=dev)
    nbd = (pdim + brick - 1) // brick
    if tri.shape[0] == 0:
        empty = torch.zeros(0, dtype=torch.int32, device=dev)
        return empty, empty
    lo = tri.min(dim=1).values.double()
    hi = tri.max(dim=1).values.double()
    plo = torch.maximum(torch.ceil(lo), torch.zeros_like(lo)).long()
    phi = torch.minimum(torch.floor(hi) + 1, (pdim - 1).double()).long()
    valid = (plo <= phi).all(dim=1)
    blo = plo // brick
    ext = torch.where(valid[:, None], phi // brick - blo + 1, torch.zeros_like(blo))
    counts = ext.prod(dim=1)
    total = int(counts.sum())
    if total >= (1 << 38):
        raise ValueError(f"{total} (triangle, brick) pairs; use a larger brick")
    # triangles within one brick (most of a fine mesh) give one pair each directly;
    # the others are expanded brick by brick
    one = counts == 1
    tid1 = torch.nonzero(one).view(-1)
    b1 = blo[tid1]
    bid1 = (b1[:, 0] * nbd[1] + b1[:, 1]) * nbd[2] + b1[:, 2]
    many = torch.nonzero(counts > 1).view(-1)
    cm = counts[many]
    nm = total - int(tid1.numel())
    k = torch.repeat_interleave(torch.arange(many.numel(), device=dev), cm)
    tidm = many[k]
    r = torch.arange(nm, device=dev) - (torch.cumsum(cm, 0) - cm)[k]
    e = ext[tidm]
    b = blo[tidm]
    bz = b[:, 2] + r % e[:, 2]
    by = b[:, 1] + (r // e[:, 2]) % e[:, 1]
    bx = b[:, 0] + r // (e[:, 2] * e[:, 1])
    bidm = (bx * nbd[1] + by) * nbd[2] + bz
    return torch.cat([tid1, tidm]).to(torch.int32), torch.cat([bid1, bidm]).to(torch.int32)


def triangles(mesh_vertices):
    """(N, 3) vertices -> (N // 3, 3, 3) float32 numpy triangles."""
    v = mesh_vertices.detach().cpu().numpy() if hasattr(mesh_vertices, "detach") else np.asarray(mesh_vertices)
    if v.shape[0] % 3:
        raise ValueError(f"{v.shape[0]} mesh vertices: a triangle soup needs a multiple of 3")
    return np.ascontiguousarray(v.astype(np.float32).reshape(-1, 3, 3))


class MeshBoundaryMasker(Operator):
    """Operator for creating a boundary missing_mask from an STL file's triangles."""

    def __init__(self, velocity_set=None, precision_policy=None, compute_backend=None, brick=8, edge_tests=False):
        super().__init__(velocity_set, precision_policy, compute_backend)
        if self.velocity_set.d == 2:
            raise NotImplementedError("This Operator is not implemented in 2D!")
        if not 1 <= int(brick) <= 1024:
            raise ValueError("brick must be in 1..1024")
        self.brick = int(brick)
        self.edge_tests = bool(edge_tests)

    def cuda_implementation(self, bc, bc_mask, missing_mask):
        name = bc.__class__.__name__
        assert bc.mesh_vertices is not None, f'Please provide the mesh vertices for {name} BC using keyword "mesh_vertices"!'
        assert bc.indices is None, f"Please use IndicesBoundaryMasker operator if {name} is imposed on known indices of the grid!"
        verts = bc.mesh_vertices
        verts = verts.detach().cpu().numpy() if hasattr(verts, "detach") else np.asarray(verts)
        assert verts.shape[1] == self.velocity_set.d, "Mesh points must be reshaped into an array (N, 3) where N indicates number of points!"
        domain_shape = tuple(int(s) for s in bc_mask.shape[1:])
        if not np.all(np.isfinite(verts)):
            raise ValueError("Mesh vertices must be finite")
        mesh_min = np.min(verts, axis=0)
        mesh_max = np.max(verts, axis=0)
        if any(mesh_min < 0) or any(mesh_max >= domain_shape):
            raise ValueError(
                f"Mesh extents ({mesh_min}, {mesh_max}) exceed domain dimensions {domain_shape}. "
                "The mesh must be fully contained within the domain."
            )
        bc.__dict__.pop("mesh_vertices", None)
        assert not bc.needs_mesh_distance, 'Please use "MeshDistanceBoundaryMasker" if this BC needs mesh distance!'
        self.apply(triangles(verts), bc.id, bc_mask, missing_mask)
        return bc_mask, missing_mask

    def apply(self, tri, bc_id, bc_mask, missing_mask):
        """Mark (bc_mask, missing_mask) in place from (T, 3, 3) triangles (numpy
        array or torch tensor, converted to float32; a pinned host tensor is
        copied to the GPU asynchronously)."""
        if bc_mask.dtype != torch.uint8 or missing_mask.dtype not in (torch.bool, torch.uint8):
            raise TypeError("bc_mask must be uint8 and missing_mask bool or uint8")
        if not (bc_mask.is_cuda and missing_mask.is_cuda and bc_mask.is_contiguous() and missing_mask.is_contiguous()):
            raise ValueError("bc_mask and missing_mask must be contiguous CUDA tensors")
        shape = tuple(int(s) for s in bc_mask.shape[1:])
        if tuple(missing_mask.shape) != (self.velocity_set.q,) + shape:
            raise ValueError("missing_mask must have shape (q, nx, ny, nz) of bc_mask's grid")
        dev = bc_mask.device
        if torch.is_tensor(tri):
            t = tri.to(device=dev, dtype=torch.float32, non_blocking=True).reshape(-1, 3, 3).contiguous()
        else:
            t = torch.as_tensor(np.asarray(tri, dtype=np.float32).reshape(-1, 3, 3), device=dev)
        pair_tri, pair_brick = brick_pairs(t, shape, self.brick)
        n_tri = int(t.shape[0])
        rec = torch.empty(max(n_tri, 1) * _lib.MESH_TRI_FLOATS, dtype=torch.float32, device=dev)
        solid = torch.empty(_lib.mesh_solid_bytes(*shape), dtype=torch.uint8, device=dev)
        tri_flat = t.reshape(-1) if n_tri else rec
        desc = make_desc(self.velocity_set, self.precision_policy, shape)
        flags = _lib.MESH_EDGE_TESTS if self.edge_tests else 0
        with torch.cuda.device(dev):
            _lib.check(
                _lib.load().xlbg_mesh_mask(
                    desc, _lib.ptr(tri_flat), n_tri, _lib.ptr(pair_tri), _lib.ptr(pair_brick), int(pair_tri.numel()),
                    self.brick, int(bc_id), flags,
                    _lib.ptr(rec), _lib.ptr(solid), _lib.ptr(bc_mask), _lib.ptr(missing_mask.view(torch.uint8)),
                    _lib.stream_handle(),
                )
            )
        _lib.mark_written(bc_mask, missing_mask)
        return bc_mask, missing_mask
