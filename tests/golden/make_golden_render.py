"""Generate golden vectors for the mesh renderer by running XLB's own
MeshRenderer source (examples/out_of_core/operators/mesh_renderer.py) on the CPU
under the Warp emulator in refshim/.

    python tests/golden/make_golden_render.py /path/to/XLB/source/tree

The emulator's ``mesh_query_ray`` is a brute-force closest hit with the
watertight ray-triangle test (Woop, Benthin and Wald, JCGT 2013), written
separately from the numpy oracle's vectorised one; everything else (camera,
rays, colour interpolation, shading, gamma, depth test) is XLB's code.  The
emulator evaluates XLB's Python-float expressions (NDC coordinates, aspect,
tan of the field of view) in float64 where Warp uses float32, so the fixtures
carry differences of a few float32 units in the last place.

Output: tests/golden/render_<case>.npz, read by tests/test_renderer.py.
"""

import importlib.util
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "refshim"))


def icosahedron(center, radius, seed):
    from scipy.spatial import ConvexHull
    from scipy.spatial.transform import Rotation

    p = (1 + 5**0.5) / 2
    v = np.array([[0, s1, s2 * p] for s1 in (-1, 1) for s2 in (-1, 1)], dtype=np.float64)
    v = np.concatenate([v, np.roll(v, 1, axis=1), np.roll(v, 2, axis=1)])
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    v = Rotation.random(random_state=seed).apply(v) * radius + np.asarray(center)
    return v, ConvexHull(v).simplices.reshape(-1)


def scene(name):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    if name == "ico_default":
        pts, ind = icosahedron((0.0, 0.0, 0.0), 0.8, 3)
        cam = dict()  # XLB's defaults: eye (0, 1, 2), target 0, up y, fov 60, ambient 0.05, sharpness 1, gamma 1
        shape = (48, 64)
    else:  # two overlapping bodies, a ground quad, custom camera and shading
        p1, i1 = icosahedron((0.3, 0.5, -0.2), 0.6, 5)
        p2, i2 = icosahedron((-0.5, 0.3, 0.4), 0.4, 9)
        quad = np.array([[-2.0, -0.2, -2.0], [2.0, -0.2, -2.0], [2.0, -0.2, 2.0], [-2.0, -0.2, 2.0]])
        qi = np.array([0, 2, 1, 0, 3, 2])
        pts = np.concatenate([p1, p2, quad])
        ind = np.concatenate([i1, i2 + len(p1), qi + len(p1) + len(p2)])
        cam = dict(camera_pos=(2.5, 1.5, 2.0), camera_target=(0.0, 0.2, 0.0), camera_up=(0.0, 1.0, 0.0),
                   fov_degrees=45.0, ambient_intensity=0.1, edge_sharpness=2.0, gamma=2.2)
        shape = (40, 72)
    colors = rng.uniform(0.1, 1.0, size=(len(pts), 3))
    depth = np.full(shape, 1.0e6, dtype=np.float32)
    depth[: shape[0] // 4, : shape[1] // 4] = 0.5  # a near plane in one corner: hits beyond it are rejected
    return pts.astype(np.float32), ind.astype(np.int32), colors.astype(np.float32), depth, cam


def run_case(name, reference_root):
    import warp as wp

    spec = importlib.util.spec_from_file_location(
        "mesh_renderer", os.path.join(reference_root, "examples", "out_of_core", "operators", "mesh_renderer.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    pts, ind, colors, depth, cam = scene(name)
    pixel = np.zeros(depth.shape + (4,), dtype=np.float32)
    depth_out = depth.copy()
    mesh = wp.Mesh(points=wp.array(pts, dtype=wp.vec3), indices=wp.array(ind, dtype=int))
    kw = {k: (wp.vec3f(*v) if isinstance(v, tuple) else v) for k, v in cam.items()}
    mod.MeshRenderer()(mesh, colors, pixel, depth_out, **kw)
    out = {"points": pts, "indices": ind, "vertex_colors": colors, "depth_in": depth, "pixel": pixel,
           "depth": depth_out}
    for k, v in cam.items():
        out["cam_" + k] = np.array(v, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), **out)
    return out


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden_render.py /path/to/XLB/source/tree [case ...]")
    import shim

    shim.install(sys.argv[1])
    for name in sys.argv[2:] or ["ico_default", "two_bodies"]:
        o = run_case(name, sys.argv[1])
        print(name, "hit pixels", int((o["pixel"][..., 3] > 0).sum()), "of", o["depth"].size, flush=True)


if __name__ == "__main__":
    main()
