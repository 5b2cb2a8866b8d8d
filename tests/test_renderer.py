"""Mesh renderer: oracle vs XLB's MeshRenderer source (golden images), the
triangle grid's lists, and the CUDA kernel vs the oracle.

Rendering is float32 arithmetic with tan and pow; the kernel uses CUDA's tanf
and powf where the oracle uses numpy's, and the golden images come from XLB's
code under an emulator that evaluates some of XLB's scalar expressions in
float64.  Tolerances (written in each test): colours 2e-5 absolute and depths
2e-5 relative on pixels where both sides hit the same face; hit masks and hit
faces equal except on at most 0.5 % of the pixels (rays that graze a triangle
edge, where a last-bit difference in the ray flips the hit).
"""

import os

import numpy as np
import pytest

from oracle import render_oracle as R

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = ["ico_default", "two_bodies"]
RGB_TOL = 2e-5
DEPTH_RTOL = 2e-5
PIXEL_FRAC = 0.005


def _golden(name):
    g = np.load(os.path.join(HERE, "golden", f"render_{name}.npz"))
    cam = {k[4:]: (tuple(g[k].tolist()) if g[k].ndim else float(g[k])) for k in g.files if k.startswith("cam_")}
    return g, cam


def _compare(pix_a, dep_a, pix_b, dep_b, face_a=None, face_b=None):
    hit_a, hit_b = pix_a[..., 3] > 0, pix_b[..., 3] > 0
    bad = hit_a != hit_b
    same = hit_a & hit_b
    if face_a is not None and face_b is not None:
        bad |= same & (face_a != face_b)
        same &= face_a == face_b
    assert bad.sum() <= PIXEL_FRAC * bad.size, f"{int(bad.sum())} of {bad.size} pixels differ in hit or face"
    assert same.sum() > 0
    drgb = np.abs(pix_a[same] - pix_b[same]).max()
    ddep = (np.abs(dep_a[same] - dep_b[same]) / np.maximum(np.abs(dep_b[same]), 1e-30)).max()
    assert drgb <= RGB_TOL, drgb
    assert ddep <= DEPTH_RTOL, ddep
    miss = ~hit_a & ~hit_b
    assert np.all(pix_a[miss] == pix_b[miss]) and np.all(dep_a[miss] == dep_b[miss])  # untouched where nothing hits


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_xlb_renderer(name):
    g, cam = _golden(name)
    pix = np.zeros(g["pixel"].shape, np.float32)
    dep = g["depth_in"].copy()
    pix, dep, _ = R.render(g["points"], g["indices"], g["vertex_colors"], pix, dep, **cam)
    _compare(pix, dep, g["pixel"], g["depth"])
    # the near plane in one corner holds: no hit beyond it
    h, w = dep.shape
    assert np.all(dep[: h // 4, : w // 4] <= 0.5)


def test_golden_images_exercise_the_renderer():
    for name in GOLDEN:
        g, _ = _golden(name)
        hit = g["pixel"][..., 3] > 0
        assert 0.1 < hit.mean() < 0.9
        assert np.unique(np.round(g["pixel"][hit][:, 0], 3)).size > 50  # shaded, not flat


def _sphere(subdiv, center=(0.0, 0.0, 0.0), radius=1.0):
    """Icosphere as (points, indices) with shared vertices."""
    p = (1 + 5**0.5) / 2
    v = [[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
         [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]]
    v = [np.array(x, float) / np.linalg.norm(x) for x in v]
    for _ in range(subdiv):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                x = v[a] + v[b]
                v.append(x / np.linalg.norm(x))
                mid[k] = len(v) - 1
            return mid[k]

        f = [g for a, b, c in f for g in ([a, m(a, b), m(c, a)], [b, m(b, c), m(a, b)], [c, m(c, a), m(b, c)],
                                          [m(a, b), m(b, c), m(c, a)])]
    pts = np.array(v) * radius + np.asarray(center)
    return pts.astype(np.float32), np.array(f, dtype=np.int32).reshape(-1)


def test_grid_lists_cover_every_candidate():
    import torch

    from xlb_gb300.operator.renderer.mesh_renderer import build_grid

    pts, ind = _sphere(2, radius=1.3)
    quad = np.array([[-2, -1, -2], [2, -1, -2], [2, -1, 2], [-2, -1, 2]], np.float32)
    pts = np.concatenate([pts, quad])
    ind = np.concatenate([ind, np.array([0, 2, 1, 0, 3, 2], np.int32) + len(pts) - 4])
    tri = torch.from_numpy(ind.astype(np.int64).reshape(-1, 3))
    g, (start, tris) = build_grid(torch.from_numpy(pts), tri, cells_per_triangle=3.0)
    start, tris = start.numpy(), tris.numpy()
    dims = np.array(list(g.dims))
    lo, cell = np.array(list(g.lo), np.float64), np.array(list(g.cell), np.float64)
    assert start[-1] == len(tris) and np.all(np.diff(start) >= 0)
    tv = pts[ind.reshape(-1, 3)].astype(np.float64)
    tlo, thi = tv.min(axis=1), tv.max(axis=1)
    assert np.all(tlo >= lo) and np.all(thi <= lo + cell * dims)
    for c in range(int(dims.prod())):
        cx, cy, cz = c // (dims[1] * dims[2]), (c // dims[2]) % dims[1], c % dims[2]
        b0 = lo + cell * np.array([cx, cy, cz])
        b1 = b0 + cell
        need = np.nonzero(np.all((tlo <= b1) & (thi >= b0), axis=1))[0]
        assert set(need.tolist()) <= set(tris[start[c]:start[c + 1]].tolist()), c


# ----------------------------------------------------------------------------- GPU


def _gpu_render(points, indices, colors, depth_in, cam, cells_per_triangle=2.0):
    import torch

    from xlb_gb300.operator.renderer import Mesh, MeshRenderer

    mesh = Mesh(points, indices, cells_per_triangle=cells_per_triangle)
    h, w = depth_in.shape
    pix = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    dep = torch.from_numpy(depth_in.copy()).cuda()
    face = torch.full((h, w), -2, dtype=torch.int32, device="cuda")
    r = MeshRenderer()
    r(mesh, colors, pix, dep, face_buffer=face, **cam)
    torch.cuda.synchronize()
    assert int(r.last_errors.item()) == 0
    return pix.cpu().numpy(), dep.cpu().numpy(), face.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN)
def test_gpu_matches_xlb_renderer_and_oracle(name):
    g, cam = _golden(name)
    pix, dep, face = _gpu_render(g["points"], g["indices"], g["vertex_colors"], g["depth_in"], cam)
    _compare(pix, dep, g["pixel"], g["depth"])
    opix = np.zeros(g["pixel"].shape, np.float32)
    odep = g["depth_in"].copy()
    opix, odep, oface = R.render(g["points"], g["indices"], g["vertex_colors"], opix, odep, **cam)
    _compare(pix, dep, opix, odep, face, oface)


@pytest.mark.gpu
@pytest.mark.parametrize("cells", [0.05, 2.0, 8.0])
def test_gpu_sphere_scene_matches_oracle(cells):
    """A 1280-triangle sphere over a ground quad, coarse to fine grids (the hit
    and its face must not depend on the grid)."""
    pts, ind = _sphere(3, center=(0.2, 0.1, -0.3), radius=0.9)
    quad = np.array([[-3, -0.8, -3], [3, -0.8, -3], [3, -0.8, 3], [-3, -0.8, 3]], np.float32)
    pts = np.concatenate([pts, quad])
    ind = np.concatenate([ind, np.array([0, 2, 1, 0, 3, 2], np.int32) + len(pts) - 4])
    colors = np.random.default_rng(6).uniform(0.1, 1.0, (len(pts), 3)).astype(np.float32)
    depth = np.full((90, 120), np.inf, np.float32)
    cam = dict(camera_pos=(1.8, 1.2, 2.4), camera_target=(0.0, 0.0, 0.0), fov_degrees=50.0, ambient_intensity=0.08,
               edge_sharpness=1.5, gamma=1.8)
    pix, dep, face = _gpu_render(pts, ind, colors, depth, cam, cells_per_triangle=cells)
    opix = np.zeros(pix.shape, np.float32)
    opix, odep, oface = R.render(pts, ind, colors, opix, depth.copy(), **cam)
    _compare(pix, dep, opix, odep, face, oface)
    assert (face >= 0).mean() > 0.3


def test_mesh_and_renderer_reject_bad_inputs():
    import torch

    from xlb_gb300.operator.renderer import Mesh, MeshRenderer

    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    with pytest.raises(ValueError, match="3 entries"):
        Mesh(pts, [0, 1], device="cpu")
    with pytest.raises(ValueError, match="outside the point array"):
        Mesh(pts, [0, 1, 3], device="cpu")
    with pytest.raises(ValueError, match="finite"):
        Mesh(np.where(pts > 0, np.nan, pts), [0, 1, 2], device="cpu")
    mesh = Mesh(pts, [0, 1, 2], device="cpu")
    assert mesh.num_triangles == 1
    r = MeshRenderer()
    with pytest.raises(TypeError):
        r((pts, [0, 1, 2]), np.ones((3, 3)), torch.zeros(4, 4, 4), torch.zeros(4, 4))
    with pytest.raises(ValueError, match="pixel_buffer"):
        r(mesh, np.ones((3, 3)), torch.zeros(4, 4, 4), torch.zeros(4, 4))  # host tensors
    with pytest.raises(ValueError, match="pixel_buffer"):
        r(mesh, np.ones((3, 3)), torch.zeros(4, 4, 3), torch.zeros(4, 4))


@pytest.mark.parametrize("case", ["empty", "single", "flat", "line"])
def test_grid_edge_cases(case):
    import torch

    from xlb_gb300.operator.renderer.mesh_renderer import build_grid

    if case == "empty":
        pts, ind = np.zeros((0, 3), np.float32), np.zeros(0, np.int64)
    elif case == "single":
        pts, ind = np.array([[0.1, 0.2, 0.3], [1.5, 0.2, 0.3], [0.1, 2.0, 0.7]], np.float32), np.arange(3)
    elif case == "flat":  # a square of 8 triangles in the plane z = 1
        g = np.stack(np.meshgrid(np.arange(3.0), np.arange(3.0), indexing="ij"), -1).reshape(-1, 2)
        pts = np.concatenate([g, np.ones((9, 1))], 1).astype(np.float32)
        ind = np.array([[i * 3 + j, i * 3 + j + 3, i * 3 + j + 1, i * 3 + j + 1, i * 3 + j + 3, i * 3 + j + 4]
                        for i in range(2) for j in range(2)]).reshape(-1)
    else:  # degenerate triangles along a line
        pts = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]], np.float32)
        ind = np.array([0, 1, 2, 1, 2, 3])
    g, (start, tris) = build_grid(torch.from_numpy(pts), torch.from_numpy(ind.reshape(-1, 3).astype(np.int64)))
    dims = list(g.dims)
    assert all(d >= 1 for d in dims) and all(c > 0 for c in g.cell)
    assert start.numel() == dims[0] * dims[1] * dims[2] + 1
    n_tri = len(ind) // 3
    assert int(start[-1]) == (0 if n_tri == 0 else tris.numel())
    if n_tri:  # every triangle is listed somewhere
        assert set(tris.tolist()) == set(range(n_tri))
