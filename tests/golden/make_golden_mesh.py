"""Generate golden vectors for the mesh boundary masker by running XLB's own
MeshBoundaryMasker source (xlb/operator/boundary_masker/mesh_boundary_masker.py)
on the CPU under the Warp emulator in refshim/.

    python tests/golden/make_golden_mesh.py /path/to/XLB/source/tree

Each case starts from a bc_mask / missing_mask with seeded prior marks (as an
indices masker would leave them), applies the mesh BCs one after the other
through XLB's operator, and stores the result twice: with the emulator's
default semantics for ``m[i][j] = x`` on a local matrix (a store into a copy of
row i, as Warp's generated code does) and with element stores that write the
matrix (``NESTED_STORES_WRITE``).  Output: tests/golden/mesh_<case>.npz, read by
tests/test_mesh_masker.py.
"""

import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "refshim"))


def box(lo, hi):
    """12 triangles of the closed box [lo, hi], (36, 3) vertices."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    c = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]])
    faces = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
             (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5), (3, 0, 4), (3, 4, 7)]
    return np.concatenate([c[list(f)] for f in faces])


def icosahedron(center, radius, seed):
    """20 triangles of a randomly rotated icosahedron, (60, 3) vertices."""
    from scipy.spatial import ConvexHull
    from scipy.spatial.transform import Rotation

    p = (1 + 5**0.5) / 2
    v = np.array([[0, s1, s2 * p] for s1 in (-1, 1) for s2 in (-1, 1)], dtype=np.float64)
    v = np.concatenate([v, np.roll(v, 1, axis=1), np.roll(v, 2, axis=1)])
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    v = Rotation.random(random_state=seed).apply(v) * radius + np.asarray(center)
    hull = ConvexHull(v)
    return np.concatenate([v[s] for s in hull.simplices])


CASES = {
    # name: (lattice, shape, [(BC class name, vertices)])
    "d3q19": ("D3Q19", (11, 10, 9), [
        ("FullwayBounceBackBC", box((2.3, 1.5, 2.0), (6.7, 5.2, 5.5))),
        ("HalfwayBounceBackBC", icosahedron((6.2, 5.9, 4.4), 2.6, 7)),
    ]),
    "d3q27": ("D3Q27", (10, 9, 8), [
        ("HalfwayBounceBackBC", np.array([
            [0.5, 0.3, 0.2], [9.4, 1.1, 6.7], [2.2, 8.6, 3.9],   # large slanted triangle
            [1.0, 1.0, 1.0], [2.0, 2.0, 2.0], [3.0, 3.0, 3.0],   # degenerate: zero normal
            [4.0, 2.0, 5.0], [7.0, 2.0, 5.0], [4.0, 6.0, 5.0],   # on integer coordinates
        ])),
    ]),
}


def run_case(name, nested_writes):
    import warp as wp
    import xlb
    from xlb.compute_backend import ComputeBackend
    from xlb.operator import boundary_condition as B
    from xlb.operator.boundary_masker import MeshBoundaryMasker
    from xlb.precision_policy import PrecisionPolicy

    wp.NESTED_STORES_WRITE = nested_writes
    lattice, shape, meshes = CASES[name]
    pp = PrecisionPolicy.FP32FP32
    vs_cls = {"D3Q19": xlb.velocity_set.D3Q19, "D3Q27": xlb.velocity_set.D3Q27}[lattice]
    vs = vs_cls(precision_policy=pp, compute_backend=ComputeBackend.WARP)
    xlb.init(velocity_set=vs, default_backend=ComputeBackend.WARP, default_precision_policy=pp)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    bc_mask = np.zeros((1,) + shape, dtype=np.uint8)
    bc_mask[0][rng.random(shape) < 0.05] = 200
    missing = rng.random((vs.q,) + shape) < 0.03
    prior = (bc_mask.copy(), missing.copy())
    bc_mask = wp.from_numpy(bc_mask)
    missing = wp.from_numpy(missing)
    masker = MeshBoundaryMasker(velocity_set=vs, precision_policy=pp, compute_backend=ComputeBackend.WARP)
    ids = []
    for cls, verts in meshes:
        bc = getattr(B, cls)(mesh_vertices=verts.copy())
        ids.append(bc.id)
        bc_mask, missing = masker(bc, bc_mask, missing)
    wp.NESTED_STORES_WRITE = False
    return prior, np.array(bc_mask), np.array(missing), ids


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden_mesh.py /path/to/XLB/source/tree [case ...]")
    import shim

    shim.install(sys.argv[1])
    for name in sys.argv[2:] or list(CASES):
        lattice, shape, meshes = CASES[name]
        prior, bm, mm, ids = run_case(name, False)
        _, bm_w, mm_w, ids_w = run_case(name, True)
        out = {"lattice": lattice, "shape": np.array(shape), "prior_bc_mask": prior[0], "prior_missing": prior[1],
               "bc_mask": bm, "missing_mask": mm, "bc_mask_edges": bm_w, "missing_mask_edges": mm_w,
               "n_mesh": len(meshes)}
        for k, (_, verts) in enumerate(meshes):
            out[f"mesh{k}_vertices"] = verts
            out[f"mesh{k}_id"] = np.array(ids[k])
            out[f"mesh{k}_id_edges"] = np.array(ids_w[k])
        np.savez_compressed(os.path.join(HERE, f"mesh_{name}.npz"), **out)
        print(name, "solid", int((bm[0] == 255).sum()), "marked", int(((bm[0] != prior[0][0]) & (bm[0] != 255)).sum()),
              "| with edge tests: solid", int((bm_w[0] == 255).sum()), flush=True)


if __name__ == "__main__":
    main()
