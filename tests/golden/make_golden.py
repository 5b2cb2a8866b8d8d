"""Generate golden vectors by running XLB's own stepper source (FP64FP64, Warp
backend code path) on the CPU under the Warp emulator in refshim/.

    python tests/golden/make_golden.py /path/to/XLB/source/tree

For each case: build XLB boundary conditions and its IncompressibleNavierStokesStepper,
call prepare_fields() (XLB's masker, equilibrium initialiser and aux-data
init), perturb f_0 with a seeded field, run a few steps with the caller swap,
and, for cases with a sphere, evaluate XLB's MomentumTransfer on the final
state.  Inputs and outputs go to tests/golden/<case>.npz.  The test
tests/test_golden.py replays every case through the oracle.
"""

import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "refshim"))

KIND_NAMES = {
    "FullwayBounceBackBC": "fullway_bb",
    "HalfwayBounceBackBC": "halfway_bb",
    "EquilibriumBC": "equilibrium",
    "ExtrapolationOutflowBC": "extrapolation",
}

CASES = {
    # name: (lattice, shape, layout, collision, omega, steps)
    "d2q9_cavity_fullway_bgk": ("D2Q9", (10, 8), "cavity_fullway", "BGK", 1.6, 3),
    "d2q9_channel_zouhe_bgk": ("D2Q9", (14, 9), "channel_zouhe", "BGK", 1.6, 3),
    "d2q9_channel_regularized_kbc": ("D2Q9", (14, 9), "channel_regularized", "KBC", 1.7, 3),
    "d3q19_cavity_fullway_bgk": ("D3Q19", (8, 7, 6), "cavity_fullway", "BGK", 1.8, 3),
    "d3q19_channel_regularized_bgk": ("D3Q19", (12, 8, 8), "channel_regularized", "BGK", 1.6, 3),
    "d3q19_channel_pressure_bgk": ("D3Q19", (10, 7, 6), "channel_pressure", "BGK", 1.6, 3),
    "d3q27_channel_regularized_kbc": ("D3Q27", (12, 8, 8), "channel_regularized", "KBC", 1.9, 2),
    "d3q27_channel_zouhe_bgk": ("D3Q27", (10, 7, 7), "channel_zouhe", "BGK", 1.5, 2),
}


def faces(grid, remove_edges):
    return grid.bounding_box_indices(remove_edges=remove_edges)


def union(*lists):
    d = len(lists[0])
    return np.unique(np.array([sum((f[i] for f in lists), []) for i in range(d)]), axis=-1).tolist()


def ball(shape, center, radius):
    g = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    r2 = sum((a - c) ** 2 for a, c in zip(g, center))
    return [list(map(int, v)) for v in np.where(r2 < radius**2)]


# Pressure values go in as 1-tuples: XLB's ZouHeBC (bc_zouhe.py:96-98) calls
# np.nonzero on the value, which numpy >= 2 rejects for a bare float; for a
# 1-tuple XLB's own handling yields the same scalar.


def build(case):
    import xlb
    import warp as wp
    from xlb.compute_backend import ComputeBackend
    from xlb.grid import grid_factory
    from xlb.operator import boundary_condition as B
    from xlb.operator.stepper import IncompressibleNavierStokesStepper
    from xlb.precision_policy import PrecisionPolicy

    lattice, shape, layout, collision, omega, steps = CASES[case]
    pp = PrecisionPolicy.FP64FP64
    vs_cls = {"D2Q9": xlb.velocity_set.D2Q9, "D3Q19": xlb.velocity_set.D3Q19, "D3Q27": xlb.velocity_set.D3Q27}[lattice]
    vs = vs_cls(precision_policy=pp, compute_backend=ComputeBackend.WARP)
    xlb.init(velocity_set=vs, default_backend=ComputeBackend.WARP, default_precision_policy=pp)
    grid = grid_factory(shape)
    d = len(shape)
    box, nob = faces(grid, False), faces(grid, True)
    side = ["bottom", "top"] if d == 2 else ["bottom", "top", "front", "back"]
    rng = np.random.default_rng(zlib.crc32(case.encode()))
    table = rng.uniform(-0.01, 0.01, size=(shape[1], shape[2] if d == 3 else 1))

    @wp.func
    def inlet(index: wp.vec3i):
        return wp.vec(wp.float64(0.04 * (1.0 + table[int(index[1]), int(index[2])])), length=1)

    center = [s // 3 if i == 0 else s // 2 for i, s in enumerate(shape)]
    radius = max(2, min(shape[1:]) // 4)
    meta = []  # (kind, value) per BC
    if layout == "cavity_fullway":
        lid_u = (0.05, 0.0) if d == 2 else (0.05, 0.0, 0.0)
        walls = union(*[box[f] for f in ["bottom", "left", "right"] + ([] if d == 2 else ["front", "back"])])
        bcs = [B.EquilibriumBC(rho=1.0, u=lid_u, indices=nob["top"]), B.FullwayBounceBackBC(indices=walls)]
        meta = [("equilibrium", 1.0, lid_u), ("fullway_bb", 0.0, None)]
        force_idx = None
    elif layout == "channel_zouhe":
        vel = (0.04,) + (0.0,) * (d - 1)
        bcs = [
            B.HalfwayBounceBackBC(indices=union(*[box[f] for f in side])),
            B.ZouHeBC("velocity", profile=inlet, indices=nob["left"]) if d == 2 else B.ZouHeBC("velocity", prescribed_value=vel, indices=nob["left"]),
            B.ZouHeBC("pressure", prescribed_value=(1.0,), indices=nob["right"]),
            B.HalfwayBounceBackBC(indices=ball(shape, center, radius)),
        ]
        meta = [("halfway_bb", 0.0, None), ("zouhe_velocity", "profile" if d == 2 else 0.04, None), ("zouhe_pressure", 1.0, None), ("halfway_bb", 0.0, None)]
        force_idx = 3
    elif layout == "channel_regularized":
        bcs = [
            B.FullwayBounceBackBC(indices=union(*[box[f] for f in side])),
            B.RegularizedBC("velocity", profile=inlet, indices=nob["left"]),
            B.ExtrapolationOutflowBC(indices=nob["right"]),
            B.HalfwayBounceBackBC(indices=ball(shape, center, radius)),
        ]
        meta = [("fullway_bb", 0.0, None), ("regularized_velocity", "profile", None), ("extrapolation", 0.0, None), ("halfway_bb", 0.0, None)]
        force_idx = 3
    elif layout == "channel_pressure":
        bcs = [
            B.HalfwayBounceBackBC(indices=union(*[box[f] for f in side])),
            B.RegularizedBC("pressure", prescribed_value=(1.005,), indices=nob["left"]),
            B.ZouHeBC("pressure", prescribed_value=(1.0,), indices=nob["right"]),
        ]
        meta = [("halfway_bb", 0.0, None), ("regularized_pressure", 1.005, None), ("zouhe_pressure", 1.0, None)]
        force_idx = None
    else:
        raise ValueError(layout)
    indices = [np.array(bc.indices, dtype=np.int64) for bc in bcs]
    stepper = IncompressibleNavierStokesStepper(grid=grid, boundary_conditions=bcs, collision_type=collision)
    return stepper, bcs, meta, indices, force_idx, table, (lattice, shape, collision, omega, steps)


def run_case(case):
    import warp as wp  # noqa: F401
    from xlb.operator.force.momentum_transfer import MomentumTransfer

    stepper, bcs, meta, indices, force_idx, table, (lattice, shape, collision, omega, steps) = build(case)
    f_0, f_1, bc_mask, missing_mask = stepper.prepare_fields()
    out = {
        "lattice": lattice, "shape": np.array(shape), "collision": collision, "omega": omega, "steps": steps,
        "profile_table": table,
        "prep_f0": np.array(f_0.numpy()), "prep_f1": np.array(f_1.numpy()),
        "bc_mask": np.array(bc_mask.numpy()), "missing_mask": np.array(missing_mask.numpy()),
        "bc_ids": np.array([bc.id for bc in bcs]), "bc_kinds": np.array([m[0] for m in meta]),
        "bc_values": np.array([m[1] if not isinstance(m[1], str) else np.nan for m in meta], dtype=np.float64),
        "bc_u": np.array([list(m[2]) + [0.0] * (3 - len(m[2])) if m[2] is not None else [0.0] * 3 for m in meta]),
    }
    for k, idx in enumerate(indices):
        out[f"bc{k}_indices"] = idx
    rng = np.random.default_rng(zlib.crc32(("perturb" + case).encode()))
    f0 = np.array(f_0.numpy())
    f0 = f0 * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, size=f0.shape))
    f_0[...] = f0
    out["in_f0"] = np.array(f_0.numpy())
    out["in_f1"] = np.array(f_1.numpy())
    for i in range(steps):
        f_0, f_1 = stepper(f_0, f_1, bc_mask, missing_mask, omega, i)
        f_0, f_1 = f_1, f_0
    out["out_f0"] = np.array(f_0.numpy())
    out["out_f1"] = np.array(f_1.numpy())
    if force_idx is not None and len(shape) == 3:  # momentum_transfer.py:103 reads c[2, l]: 3D only
        mt = MomentumTransfer(bcs[force_idx])
        out["force_bc_id"] = np.array(bcs[force_idx].id)
        out["force"] = np.array(mt(f_0, f_1, bc_mask, missing_mask), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, f"{case}.npz"), **out)
    return out


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py /path/to/XLB/source/tree [case ...]")
    import shim

    shim.install(sys.argv[1])
    cases = sys.argv[2:] or list(CASES)
    for case in cases:
        o = run_case(case)
        print(case, "steps", int(o["steps"]), "force" if "force" in o else "", flush=True)


if __name__ == "__main__":
    main()
