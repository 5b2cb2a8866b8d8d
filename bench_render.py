"""Mesh renderer timing: a 1920 x 1080 frame of the wind-tunnel body.

The body is bench_mesh.py's ellipsoid (semi-axes 64, 24, 20 cells, ``--subdiv``
midpoint subdivisions of an icosahedron: 8 gives 1 310 720 triangles) as a
triangle soup with a vertex colour per corner, seen from a three-quarter view
with XLB's MeshRenderer defaults for shading.  Times (CUDA events): the first
call, which builds the triangle grid, and then ``--reps`` frames, each resetting
the depth buffer and rendering.  Prints one JSON line.
"""

import argparse
import json

import numpy as np
import torch

from bench_mesh import ellipsoid


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--subdiv", type=int, default=8)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--cells", type=float, default=2.0, help="grid cells per triangle")
    args = ap.parse_args()

    from xlb_gb300.operator.renderer import Mesh, MeshRenderer

    tri = ellipsoid(args.subdiv, (192.0, 64.0, 21.0), (64.0, 24.0, 20.0)).astype(np.float32)
    pts = tri.reshape(-1, 3)
    ind = np.arange(len(pts), dtype=np.int32)
    colors = (0.5 + 0.5 * (pts - pts.min(0)) / (pts.max(0) - pts.min(0))).astype(np.float32)
    h, w = args.height, args.width
    pix = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    dep = torch.full((h, w), float("inf"), dtype=torch.float32, device="cuda")
    cam = dict(camera_pos=(330.0, 180.0, 120.0), camera_target=(192.0, 64.0, 21.0), camera_up=(0.0, 0.0, 1.0),
               fov_degrees=40.0)
    render = MeshRenderer()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mesh = Mesh(pts, ind, cells_per_triangle=args.cells)
    torch.cuda.synchronize()
    e0.record()
    render(mesh, colors, pix, dep, **cam)  # builds the grid
    e1.record()
    torch.cuda.synchronize()
    first_ms = e0.elapsed_time(e1)
    for _ in range(3):
        dep.fill_(float("inf"))
        render(mesh, colors, pix, dep, **cam)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.reps):
        dep.fill_(float("inf"))
        render(mesh, colors, pix, dep, **cam)
    e1.record()
    torch.cuda.synchronize()
    frame_ms = e0.elapsed_time(e1) / args.reps
    g, _ = mesh.grid()
    print(json.dumps({
        "workload": f"mesh renderer, {w}x{h}, ellipsoid body 128x48x40, {mesh.num_triangles} triangles",
        "triangles": mesh.num_triangles, "grid_dims": list(g.dims), "first_call_ms": round(first_ms, 2),
        "frame_ms": round(frame_ms, 3), "mrays_per_s": round(h * w / (frame_ms * 1e3), 1),
        "hit_fraction": round(float((pix[..., 3] > 0).float().mean()), 4),
        "errors": int(render.last_errors.item()),
    }))


if __name__ == "__main__":
    main()
