"""Mesh boundary masker timing on the 3D wind-tunnel set-up.

Grid 512 x 128 x 128 with D3Q27, the shape and lattice of XLB's
examples/cfd/windtunnel_3d.py, and a closed body of the size that example gives
its car (length grid_x / 4 = 128 cells, resting on the floor, centred in y):
a triangulated ellipsoid with semi-axes (64, 24, 20) made by ``--subdiv``
midpoint subdivisions of an icosahedron (8: 1 310 720 triangles, about the
size of a detailed car surface mesh).  The masker runs after an indices-style
prior marking of the tunnel walls; times are CUDA-event times over ``--reps``
repetitions after ``--warmup``:

* ``apply_ms``: MeshBoundaryMasker.apply as a stepper calls it: triangle upload
  from host memory, the (triangle, brick) work list (torch ops on the
  device), the kernels;
* ``kernels_ms``: the C-ABI call alone (flag reset, precompute, solid flags,
  marks) with the (triangle, brick) work list built.

Prints one JSON line.
"""

import argparse
import json
import time

import numpy as np
import torch


def ellipsoid(subdiv, center, axes):
    """Triangle soup (T, 3, 3) of an ellipsoid from a subdivided icosahedron."""
    p = (1 + 5**0.5) / 2
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    t = v[f]
    t /= np.linalg.norm(t, axis=2, keepdims=True)
    for _ in range(subdiv):
        a, b, c = t[:, 0], t[:, 1], t[:, 2]
        ab, bc, ca = (a + b), (b + c), (c + a)
        ab, bc, ca = (x / np.linalg.norm(x, axis=1, keepdims=True) for x in (ab, bc, ca))
        t = np.stack([np.stack(s, axis=1) for s in ((a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca))], axis=1)
        t = t.reshape(-1, 3, 3)
    return t * np.asarray(axes) + np.asarray(center)


def _time(fn, reps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", type=int, nargs=3, default=[512, 128, 128])
    ap.add_argument("--subdiv", type=int, default=8)
    ap.add_argument("--brick", type=int, default=8)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args()

    import xlb_gb300 as xlb
    from xlb_gb300 import _lib
    from xlb_gb300.operator.boundary_masker import MeshBoundaryMasker
    from xlb_gb300.operator.boundary_masker.mesh_boundary_masker import brick_pairs
    from xlb_gb300.operator.stepper.desc import make_desc

    shape = tuple(args.shape)
    pp = xlb.PrecisionPolicy.FP32FP32
    vs = xlb.velocity_set.D3Q27(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    nx, ny, nz = shape
    t0 = time.perf_counter()
    tri = ellipsoid(args.subdiv, (nx / 4 + 64, ny / 2, 21.0), (64.0, 24.0, 20.0)).astype(np.float32)
    gen_s = time.perf_counter() - t0
    tri_host = torch.from_numpy(np.ascontiguousarray(tri)).pin_memory()

    dev = torch.device("cuda:0")
    bc_mask = torch.zeros((1,) + shape, dtype=torch.uint8, device=dev)
    bc_mask[0, :, 0, :] = 1
    bc_mask[0, :, -1, :] = 1
    bc_mask[0, :, :, 0] = 1
    bc_mask[0, :, :, -1] = 1
    missing = torch.zeros((vs.q,) + shape, dtype=torch.bool, device=dev)
    prior = (bc_mask.clone(), missing.clone())
    masker = MeshBoundaryMasker(vs, pp, brick=args.brick)

    def apply():
        masker.apply(tri_host, 4, bc_mask, missing)

    apply_ms = _time(apply, args.reps, args.warmup)

    t = tri_host.to(dev)
    pair_tri, pair_brick = brick_pairs(t, shape, args.brick)
    n_tri = int(t.shape[0])
    rec = torch.empty(n_tri * _lib.MESH_TRI_FLOATS, dtype=torch.float32, device=dev)
    solid = torch.empty(_lib.mesh_solid_bytes(nx, ny, nz), dtype=torch.uint8, device=dev)
    desc = make_desc(vs, pp, shape)
    lib = _lib.load()
    stream = _lib.stream_handle()
    args_c = (desc, _lib.ptr(t.reshape(-1)), n_tri, _lib.ptr(pair_tri), _lib.ptr(pair_brick), int(pair_tri.numel()),
              args.brick, 4, 0, _lib.ptr(rec), _lib.ptr(solid), _lib.ptr(bc_mask), _lib.ptr(missing.view(torch.uint8)),
              stream)

    def kernels():
        _lib.check(lib.xlbg_mesh_mask(*args_c))

    kernels_ms = _time(kernels, args.reps, args.warmup)

    # the result is the same however often it is applied
    bc_mask.copy_(prior[0])
    missing.copy_(prior[1])
    kernels()
    torch.cuda.synchronize()
    n_solid = int((bc_mask == 255).sum())
    n_marked = int((bc_mask == 4).sum())
    pairs = int(pair_tri.numel())
    voxels = (nx + 2) * (ny + 2) * (nz + 2)
    print(json.dumps({
        "workload": f"mesh masker, D3Q27 {nx}x{ny}x{nz}, ellipsoid body 128x48x40 cells, {n_tri} triangles",
        "triangles": n_tri, "brick": args.brick, "brick_triangle_pairs": pairs,
        "padded_voxels": voxels, "solid_voxels": n_solid, "marked_cells": n_marked,
        "apply_ms": round(apply_ms, 3), "kernels_ms": round(kernels_ms, 3),
        "voxels_per_s": voxels / (kernels_ms * 1e-3), "host_mesh_generation_s": round(gen_s, 2),
        "gpu_launches_per_apply": 3,
    }))


if __name__ == "__main__":
    main()
