"""Shared set-ups: the same boundary layout built through xlb_gb300 (GPU) and the oracle (CPU).

Used by the parity tests only; the oracle is the checker here.
"""

import numpy as np

from oracle import lbm_oracle as O

POLICIES = {
    "fp32": ("FP32FP32", "f32", np.float32),
    "fp64": ("FP64FP64", "f64", np.float64),
    "f16": ("FP32FP16", "f16", np.float32),
    "f16s": ("FP32FP16S", "f16s", np.float32),
    "bf16s": ("FP32BF16S", "bf16s", np.float32),
    "f16sr": ("FP32FP16SR", "f16s", np.float32),
    "bf16sr": ("FP32BF16SR", "bf16s", np.float32),
    "fp64f32": ("FP64FP32", "f32", np.float64),
    "fp64f16": ("FP64FP16", "f16", np.float64),
}


def faces(shape, remove_edges):
    from xlb_gb300.grid import grid_factory

    return grid_factory(shape, device="cpu").bounding_box_indices(remove_edges=remove_edges)


def union(*face_lists):
    d = len(face_lists[0])
    cat = [sum((f[i] for f in face_lists), []) for i in range(d)]
    return np.unique(np.array(cat), axis=-1).tolist()


def ball(shape, center, radius):
    grids = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    r2 = sum((g - c) ** 2 for g, c in zip(grids, center))
    idx = np.where(r2 < radius**2)
    return [list(map(int, v)) for v in idx]


def inlet_profile(shape, u0=0.04, seed=7):
    """Seeded +-1 % per-cell perturbation of u0; a function of the cell index only."""
    pert = np.random.default_rng(seed).uniform(-0.01, 0.01, size=tuple(shape) + ((1,) if len(shape) == 2 else ()))

    def profile(idx3):
        return u0 * (1.0 + pert[idx3[0], idx3[1], idx3[2]])

    return profile


def layout(name, shape):
    """[(kind, indices, params)] for a named boundary layout."""
    d = len(shape)
    box = faces(shape, False)
    nob = faces(shape, True)
    lid_u = (0.05, 0.0) if d == 2 else (0.05, 0.0, 0.0)
    side = ["bottom", "top"] if d == 2 else ["bottom", "top", "front", "back"]
    center = [s // 3 if i == 0 else s // 2 for i, s in enumerate(shape)]
    radius = max(2, min(shape[1:]) // 5)
    if name == "periodic":
        return []
    if name in ("cavity_fullway", "cavity_halfway"):
        wall_faces = ["bottom", "left", "right"] + ([] if d == 2 else ["front", "back"])
        walls = union(*[box[f] for f in wall_faces])
        kind = "fullway_bb" if name == "cavity_fullway" else "halfway_bb"
        return [("equilibrium", nob["top"], {"rho": 1.0, "u": lid_u}), (kind, walls, {})]
    if name == "channel_zouhe":
        return [
            ("halfway_bb", union(*[box[f] for f in side]), {}),
            ("zouhe_velocity", nob["left"], {"profile": inlet_profile(shape)}),
            ("zouhe_pressure", nob["right"], {"value": 1.0}),
            ("halfway_bb", ball(shape, center, radius), {}),
        ]
    if name == "channel_regularized":
        return [
            ("fullway_bb", union(*[box[f] for f in side]), {}),
            ("regularized_velocity", nob["left"], {"profile": inlet_profile(shape)}),
            ("extrapolation", nob["right"], {}),
            ("halfway_bb", ball(shape, center, radius), {}),
        ]
    if name == "channel_pressure":
        return [
            ("halfway_bb", union(*[box[f] for f in side]), {}),
            ("regularized_pressure", nob["left"], {"value": 1.005}),
            ("zouhe_pressure", nob["right"], {"value": 1.0}),
        ]
    raise ValueError(name)


def make_xlb_bc(kind, indices, params):
    from xlb_gb300.operator import boundary_condition as B

    if kind == "fullway_bb":
        return B.FullwayBounceBackBC(indices=indices)
    if kind == "halfway_bb":
        return B.HalfwayBounceBackBC(indices=indices)
    if kind == "equilibrium":
        return B.EquilibriumBC(rho=params["rho"], u=params["u"], indices=indices)
    if kind == "extrapolation":
        return B.ExtrapolationOutflowBC(indices=indices)
    cls = B.ZouHeBC if kind.startswith("zouhe") else B.RegularizedBC
    bc_type = "velocity" if kind.endswith("velocity") else "pressure"
    if "profile" in params:
        return cls(bc_type, profile=params["profile"], indices=indices)
    if bc_type == "velocity":
        return cls(bc_type, prescribed_value=(params["value"],) + (0.0,) * (len(indices) - 1), indices=indices)
    return cls(bc_type, prescribed_value=params["value"], indices=indices)


class Scenario:
    """Holds both sides of one set-up."""

    def __init__(self, lattice, shape, layout_name, policy="fp32", collision="BGK", omega=1.6):
        import xlb_gb300 as xlb
        from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

        pname, skind, T = POLICIES[policy]
        self.T = T
        self.omega = omega
        # shifted FP16/BF16 policies run BGK on the stored deviations (the stepper picks it),
        # their SR variants with stochastic rounding of the stores
        self.collision = collision
        if collision == "BGK" and pname in ("FP32FP16S", "FP32BF16S"):
            self.collision = "BGK_SHIFTED"
        if collision in ("BGK", "BGK_SHIFTED") and pname in ("FP32FP16SR", "FP32BF16SR"):
            self.collision = "BGK_SHIFTED_SR"
        self.lat = O.Lattice(lattice)
        self.store = O.Store(skind, self.lat)
        self.shape = tuple(shape)
        vs_cls = {"D2Q9": xlb.velocity_set.D2Q9, "D3Q19": xlb.velocity_set.D3Q19, "D3Q27": xlb.velocity_set.D3Q27}[lattice]
        pp = getattr(xlb.PrecisionPolicy, pname)
        xlb.init(vs_cls(pp), xlb.ComputeBackend.CUDA, pp)
        spec = layout(layout_name, shape)
        self.xbcs = [make_xlb_bc(k, idx, p) for k, idx, p in spec]
        self.obcs = [
            O.BC(k, bc.id, idx, rho=p.get("rho", 1.0), u=p.get("u", (0, 0, 0)), value=getattr(bc, "prescribed_value", None),
                 profile=p.get("profile"))
            for (k, idx, p), bc in zip(spec, self.xbcs)
        ]
        self.grid = xlb.grid.grid_factory(shape)
        self.stepper = IncompressibleNavierStokesStepper(self.grid, self.xbcs, collision_type=collision)
        # oracle side of prepare_fields
        self.bc_mask, self.missing = O.masker(self.lat, shape, self.obcs)
        f0 = O.initial_equilibrium(self.lat, self.store, shape, T)
        self.f0 = f0
        self.f1 = O.aux_init(self.lat, self.store, f0.copy(), self.bc_mask, self.missing, self.obcs, T)

    def randomize(self, seed=0, amp=0.05):
        """Perturb the oracle state around rest equilibrium (same for both sides after upload)."""
        rng = np.random.default_rng(seed)
        s3 = self.f0.shape[1:]
        w = self.lat.w.reshape((-1,) + (1,) * len(s3))
        f = (w * (1.0 + amp * rng.uniform(-1, 1, size=(self.lat.q,) + s3))).astype(self.T)
        self.f0 = self.store.encode(f, self.T)
        self.f1 = O.aux_init(self.lat, self.store, self.f0.copy(), self.bc_mask, self.missing, self.obcs, self.T)

    def oracle_steps(self, steps):
        with np.errstate(all="ignore"):
            return O.run(self.lat, self.store, self.f0.copy(), self.f1.copy(), self.bc_mask, self.missing, self.omega,
                         self.obcs, steps, self.collision, self.T)

    # ---------------------------------------------------------------- GPU side
    def to_torch(self, arr):
        import torch

        if self.store.kind == "bf16s":
            return torch.from_numpy(arr.view(np.int16).copy()).view(torch.bfloat16).cuda()
        return torch.from_numpy(np.ascontiguousarray(arr)).cuda()

    def to_numpy(self, t):
        import torch

        t = t.detach().cpu()
        if self.store.kind == "bf16s":
            return t.view(torch.int16).numpy().view(np.uint16)
        return t.numpy()

    def gpu_fields(self):
        """Upload the oracle state and masks; returns (f_0, f_1, bc_mask, missing_mask)."""
        import torch

        return (
            self.to_torch(self.f0),
            self.to_torch(self.f1),
            torch.from_numpy(self.bc_mask).cuda(),
            torch.from_numpy(self.missing).cuda(),
        )

    def gpu_steps(self, steps, use_run=False):
        import torch

        f_0, f_1, bcm, mm = self.gpu_fields()
        if use_run:
            f_0, f_1 = self.stepper.run(f_0, f_1, bcm, mm, self.omega, steps)
        else:
            for i in range(steps):
                f_0, f_1 = self.stepper(f_0, f_1, bcm, mm, self.omega, i)
                f_0, f_1 = f_1, f_0
        torch.cuda.synchronize()
        return self.to_numpy(f_0), self.to_numpy(f_1)
