"""Ray-traced mesh renderer (XLB's out-of-core example operator
examples/out_of_core/operators/mesh_renderer.py:5-245).

``MeshRenderer()(mesh, vertex_colors, pixel_buffer, depth_buffer, camera_pos,
camera_target, camera_up, fov_degrees, ambient_intensity, edge_sharpness,
gamma)`` with XLB's defaults renders into a (height, width, 4) RGBA float32
buffer and a (height, width) depth buffer (CUDA tensors): per pixel the closest
hit with t below the depth already there, vertex colours interpolated with the
hit's barycentrics, normal-based shading and gamma, written on a hit only.  The
work is the CUDA kernel of ``xlbg_render_mesh``.

XLB passes a ``wp.Mesh`` (points, indices, BVH); here ``Mesh(points, indices)``
holds the same arrays on the GPU and, built on first use, a uniform grid of
triangle lists that the kernel walks instead of a BVH.  The hit is the
watertight ray-triangle test's (Woop, Benthin and Wald, JCGT 2013); among
equal t the lowest face index wins, where Warp's choice depends on its BVH.
"""

import ctypes

import numpy as np
import torch

from xlb_gb300 import _lib


class Mesh:
    """Triangle mesh on the GPU: points (N, 3) float32, indices (3T,) int32
    (triangle t is indices[3t : 3t + 3], as in ``wp.Mesh``)."""

    def __init__(self, points, indices, device="cuda", cells_per_triangle=2.0):
        self.points = torch.as_tensor(np.asarray(points, dtype=np.float32) if not torch.is_tensor(points) else points,
                                      dtype=torch.float32, device=device).reshape(-1, 3).contiguous()
        ind = indices if torch.is_tensor(indices) else torch.as_tensor(np.asarray(indices).astype(np.int64))
        ind = ind.to(device=device, dtype=torch.int64).reshape(-1)
        if ind.numel() % 3:
            raise ValueError("indices must hold 3 entries per triangle")
        if ind.numel() and (int(ind.min()) < 0 or int(ind.max()) >= self.points.shape[0]):
            raise ValueError("mesh indices outside the point array")
        if not bool(torch.isfinite(self.points).all()):
            raise ValueError("mesh points must be finite")
        self.indices = ind.to(torch.int32).contiguous()
        self.cells_per_triangle = float(cells_per_triangle)
        self._grid = None

    @property
    def num_triangles(self):
        return self.indices.numel() // 3

    def grid(self):
        """(xlbg_tri_grid, keep-alive tensors), built once."""
        if self._grid is None:
            self._grid = build_grid(self.points, self.indices.reshape(-1, 3).long(), self.cells_per_triangle)
        return self._grid


def build_grid(points, tri_index, cells_per_triangle=2.0, max_dim=1024):
    """Uniform grid over the mesh bounds with about ``cells_per_triangle`` cells
    per triangle; lists, per cell, every triangle whose bounds (widened by 1e-4
    of a cell) meet the cell.  Returns (xlbg_tri_grid, (cell_start, cell_tris))."""
    dev = points.device
    n_tri = tri_index.shape[0]
    if n_tri == 0:
        start = torch.zeros(2, dtype=torch.int32, device=dev)
        tris = torch.zeros(1, dtype=torch.int32, device=dev)
        g = _lib.TriGrid()
        g.lo[:] = [0.0, 0.0, 0.0]
        g.cell[:] = [1.0, 1.0, 1.0]
        g.dims[:] = [1, 1, 1]
        g.cell_start = ctypes.c_void_p(start.data_ptr())
        g.cell_tris = ctypes.c_void_p(tris.data_ptr())
        return g, (start, tris)
    p = points.double()
    lo = p.min(dim=0).values
    hi = p.max(dim=0).values
    ext = hi - lo
    pad = 1e-3 * max(float(ext.max()), 1e-6)
    lo = lo - pad
    hi = hi + pad
    ext = hi - lo
    target = max(1.0, min(cells_per_triangle * n_tri, float(1 << 24)))
    h = (float(ext.prod()) / target) ** (1.0 / 3.0)
    dims = torch.clamp(torch.ceil(ext / h), 1, max_dim).long()
    lo32 = lo.float()
    cell32 = (ext / dims.double()).float()
    # per-triangle cell ranges, in the kernel's float32 cell boundaries, widened
    tri = p[tri_index]  # (T, 3, 3)
    tlo = tri.min(dim=1).values
    thi = tri.max(dim=1).values
    c = cell32.double()
    l32 = lo32.double()
    c0 = torch.clamp(torch.floor((tlo - l32) / c - 1e-4), min=0).long()
    c1 = torch.minimum(torch.floor((thi - l32) / c + 1e-4).long(), dims - 1)
    c0 = torch.minimum(c0, dims - 1)
    ext_c = c1 - c0 + 1
    counts = ext_c.prod(dim=1)
    total = int(counts.sum())
    if total >= (1 << 31) - 1:
        raise ValueError(f"{total} (cell, triangle) entries; use fewer cells")
    tid = torch.repeat_interleave(torch.arange(n_tri, device=dev), counts)
    r = torch.arange(total, device=dev) - (torch.cumsum(counts, 0) - counts)[tid]
    e = ext_c[tid]
    b = c0[tid]
    cz = b[:, 2] + r % e[:, 2]
    cy = b[:, 1] + (r // e[:, 2]) % e[:, 1]
    cx = b[:, 0] + r // (e[:, 2] * e[:, 1])
    cid = (cx * dims[1] + cy) * dims[2] + cz
    order = torch.argsort(cid, stable=True)
    tris = tid[order].to(torch.int32).contiguous()
    ncell = int(dims.prod())
    start = torch.zeros(ncell + 1, dtype=torch.int64, device=dev)
    start[1:] = torch.cumsum(torch.bincount(cid, minlength=ncell), 0)
    start = start.to(torch.int32).contiguous()
    g = _lib.TriGrid()
    g.lo[:] = [float(v) for v in lo32.tolist()]
    g.cell[:] = [float(v) for v in cell32.tolist()]
    g.dims[:] = [int(v) for v in dims.tolist()]
    g.cell_start = ctypes.c_void_p(start.data_ptr())
    g.cell_tris = ctypes.c_void_p(tris.data_ptr())
    return g, (start, tris)


def _vec(v):
    if hasattr(v, "detach"):
        v = v.detach().cpu().numpy()
    return [float(x) for x in np.asarray(v, dtype=np.float64).reshape(3)]


class MeshRenderer:
    """Render a mesh to a pixel and depth buffer with ray tracing and
    normal-based shading (XLB's MeshRenderer, same call and defaults)."""

    def __call__(self, mesh, vertex_colors, pixel_buffer, depth_buffer, camera_pos=(0.0, 1.0, 2.0),
                 camera_target=(0.0, 0.0, 0.0), camera_up=(0.0, 1.0, 0.0), fov_degrees=60.0, ambient_intensity=0.05,
                 edge_sharpness=1.0, gamma=1.0, face_buffer=None):
        if not isinstance(mesh, Mesh):
            raise TypeError("mesh must be an xlb_gb300 Mesh(points, indices)")
        h, w = int(depth_buffer.shape[0]), int(depth_buffer.shape[1])
        for name, t, shape in (("pixel_buffer", pixel_buffer, (h, w, 4)), ("depth_buffer", depth_buffer, (h, w))):
            if tuple(t.shape) != shape or t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous float32 CUDA tensor of shape {shape}")
        colors = torch.as_tensor(vertex_colors, dtype=torch.float32, device=pixel_buffer.device).reshape(-1, 3)
        colors = colors.contiguous()
        if colors.shape[0] != mesh.points.shape[0]:
            raise ValueError("vertex_colors must have one RGB row per mesh point")
        if face_buffer is not None and (tuple(face_buffer.shape) != (h, w) or face_buffer.dtype != torch.int32
                                        or not face_buffer.is_cuda or not face_buffer.is_contiguous()):
            raise ValueError("face_buffer must be a contiguous int32 CUDA tensor of shape (height, width)")
        grid, _ = mesh.grid()  # the list tensors stay alive in the mesh
        cam = _lib.Camera()
        cam.eye[:] = _vec(camera_pos)
        cam.target[:] = _vec(camera_target)
        cam.up[:] = _vec(camera_up)
        cam.fov_degrees = float(fov_degrees)
        cam.ambient_intensity = float(ambient_intensity)
        cam.edge_sharpness = float(edge_sharpness)
        cam.gamma = float(gamma)
        err = torch.zeros(1, dtype=torch.int32, device=pixel_buffer.device)
        with torch.cuda.device(pixel_buffer.device):
            _lib.check(
                _lib.load().xlbg_render_mesh(
                    _lib.ptr(mesh.points), int(mesh.points.shape[0]), _lib.ptr(mesh.indices), mesh.num_triangles,
                    _lib.ptr(colors), ctypes.byref(grid), ctypes.byref(cam), h, w, _lib.ptr(pixel_buffer),
                    _lib.ptr(depth_buffer), _lib.ptr(face_buffer), _lib.ptr(err), _lib.stream_handle(),
                )
            )
        self.last_errors = err  # skipped malformed list entries (0 for lists built by Mesh)
        return pixel_buffer, depth_buffer
