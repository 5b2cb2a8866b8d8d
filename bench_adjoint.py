"""Differentiation workload: a channel with a learnable inlet profile, the
gradient through the checkpointed hand-written adjoint, and its cost.

Set-up, in 2D (D2Q9, 512 x 128) or 3D (D3Q19, 128^3):
* obstacle: the cells where a sum of 8 seeded Gaussian bumps exceeds 0.5,
  voxelised as HalfwayBounceBack; HalfwayBounceBack walls on the faces
  normal to y (and z in 3D);
* ZouHe velocity inlet on x = 0 with a parabolic profile, peak 0.05, scaled by
  a learnable amplitude per y-row; ZouHe pressure outlet (rho = 1) on x = nx-1;
* BGK, omega = 1.6, initial state rest equilibrium;
* loss: mean squared difference between the final velocity field and that
  of a target run whose amplitudes are 1 + 0.1 sin(2 pi y / ny) (seeded data);
* gradient with respect to the initial populations and the per-row
  amplitudes, checkpoints every 100 steps.

Reported: forward and backward time (CUDA events), their ratio, peak device
memory, and the gradient error against FP64 central finite differences along
a seeded random direction of the amplitudes (FP64FP64 runs), for the FP32
adjoint (forward as BGK on deviations from rest, collision_type "BGK_SHIFTED";
and with XLB's BGK order for comparison) and for the FP64 adjoint.

Run directly (``python bench_adjoint.py --dim 2``) for one JSON line, or call
``measure`` from bench.py.
"""

import argparse
import json
import math

import numpy as np
import torch


def _build(dim, policy_name, steps, collision="BGK"):
    import xlb_gb300 as xlb
    from xlb_gb300.operator import boundary_condition as B
    from xlb_gb300.operator.boundary_condition import boundary_condition_registry as reg
    from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

    # fresh BC ids for every build (ids are global and never reused otherwise)
    reg.id_to_bc.clear()
    reg.bc_to_id.clear()
    reg.next_id = 1
    shape = (512, 128) if dim == 2 else (128, 128, 128)
    pp = getattr(xlb.PrecisionPolicy, policy_name)
    vs = (xlb.velocity_set.D2Q9 if dim == 2 else xlb.velocity_set.D3Q19)(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    grid = xlb.grid.grid_factory(shape)
    box = grid.bounding_box_indices(remove_edges=False)
    nob = grid.bounding_box_indices(remove_edges=True)
    rng = np.random.default_rng(2024)
    g = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    field = np.zeros(shape)
    for _ in range(8):
        c = [rng.uniform(0.2, 0.6) * shape[0]] + [rng.uniform(0.25, 0.75) * s for s in shape[1:]]
        sig = rng.uniform(3.0, 7.0) * (shape[1] / 128.0)
        field += rng.uniform(0.6, 1.0) * np.exp(-sum((gi - ci) ** 2 for gi, ci in zip(g, c)) / (2 * sig**2))
    obst = [list(map(int, v)) for v in np.nonzero(field > 0.5)]
    walls_faces = ["bottom", "top"] if dim == 2 else ["bottom", "top", "front", "back"]
    walls = np.unique(np.concatenate([np.array(box[f]) for f in walls_faces], axis=1), axis=1).tolist()
    bcs = [
        B.HalfwayBounceBackBC(indices=walls),
        B.ZouHeBC("velocity", prescribed_value=(0.05,) + (0.0,) * (dim - 1), indices=nob["left"]),
        B.ZouHeBC("pressure", prescribed_value=1.0, indices=nob["right"]),
        B.HalfwayBounceBackBC(indices=obst),
    ]
    stepper = IncompressibleNavierStokesStepper(grid, bcs, collision_type=collision)
    f_0, f_1, bc_mask, missing = stepper.prepare_fields()
    run = stepper.differentiable(bc_mask, missing, 1.6, steps, checkpoint_every=100)
    # prescribed values as prepare_fields stored them (outlet density 1 stays);
    # the learnable part is the inlet: its cells, their y-row, the parabola
    base = run.aux_from_fields(f_1)
    ids_at = bc_mask.view(-1)[run.aux_cells]
    inlet_sel = torch.nonzero(ids_at == bcs[1].id).view(-1)
    cells = run.aux_cells[inlet_sel].cpu().numpy()
    idx = np.array(np.unravel_index(cells, tuple(bc_mask.shape[1:])))
    ny = shape[1]
    rows = idx[1]
    yy = (rows - 0.5) / (ny - 2)
    para = 4.0 * yy * (1.0 - yy)
    if dim == 3:
        zz = (idx[2] - 0.5) / (shape[2] - 2)
        para = para * 4.0 * zz * (1.0 - zz)
    dev = f_0.device
    ctx = {
        "stepper": stepper, "run": run, "f_0": f_0, "bc_mask": bc_mask, "shape": shape, "base": base,
        "inlet_sel": inlet_sel,
        "rows": torch.as_tensor(rows, device=dev), "para": torch.as_tensor(0.05 * para, device=dev), "ny": ny,
        "fluid": (bc_mask[0] == 0).to(pp.compute_precision.torch_dtype),
    }
    return ctx


def _velocity(f, c):
    rho = f.sum(0)
    return torch.einsum("dq,q...->d...", c, f) / rho


def _aux(ctx, amp):
    """All prescribed values, with the inlet's set from the per-row amplitudes."""
    inlet = ctx["para"].to(amp.dtype) * amp[ctx["rows"]]
    return ctx["base"].to(amp.dtype).scatter(0, ctx["inlet_sel"], inlet)


def _loss_fn(ctx, c, u_target):
    def loss(f_init, amp):
        f = ctx["run"](f_init, _aux(ctx, amp))
        u = _velocity(f.to(amp.dtype), c)
        return (((u - u_target) ** 2) * ctx["fluid"].to(amp.dtype)).sum() / ctx["fluid"].sum()

    return loss


def _c_matrix(stepper, dtype, device):
    c = np.asarray(stepper.velocity_set.c, dtype=np.float64)  # (d, q)
    return torch.as_tensor(c, dtype=dtype, device=device)


def measure_fp32(dim=2, steps=None):
    """The FP32 forward + backward only (target from an FP32 run), for profiling."""
    steps = steps or (2000 if dim == 2 else 500)
    dev = torch.device("cuda")
    ctx = _build(dim, "FP32FP32", steps, collision="BGK_SHIFTED")
    ny = ctx["ny"]
    y = torch.arange(ny, dtype=torch.float32, device=dev)
    c32 = _c_matrix(ctx["stepper"], torch.float32, dev)
    with torch.no_grad():
        u_target = _velocity(ctx["run"](ctx["f_0"], _aux(ctx, 1.0 + 0.1 * torch.sin(2 * math.pi * y / ny))), c32)
    loss = _loss_fn(ctx, c32, u_target)
    times = []
    for _ in range(2):  # warm-up, timed
        amp = torch.ones(ny, dtype=torch.float32, device=dev, requires_grad=True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record()
        L = loss(ctx["f_0"].clone().requires_grad_(True), amp)
        e1.record()
        L.backward()
        e2.record()
        torch.cuda.synchronize()
        times.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
    return {"steps": steps, "fwd_ms": times[-1][0], "bwd_ms": times[-1][1],
            "adjoint_to_forward": times[-1][1] / times[-1][0]}


def measure(dim=2, steps=None, h=1e-5, fd=True):
    """One differentiation run; returns a dict of the reported figures."""
    steps = steps or (2000 if dim == 2 else 500)
    dev = torch.device("cuda")
    # FP64 side: the target field and the finite-difference reference
    ctx64 = _build(dim, "FP64FP64", steps)
    ny = ctx64["ny"]
    y = torch.arange(ny, dtype=torch.float64, device=dev)
    amp_target = 1.0 + 0.1 * torch.sin(2 * math.pi * y / ny)
    c64 = _c_matrix(ctx64["stepper"], torch.float64, dev)
    with torch.no_grad():
        f_t = ctx64["run"](ctx64["f_0"], _aux(ctx64, amp_target))
        u_target = _velocity(f_t, c64)
    loss64 = _loss_fn(ctx64, c64, u_target)
    amp64 = torch.ones(ny, dtype=torch.float64, device=dev, requires_grad=True)
    f64 = ctx64["f_0"].clone().requires_grad_(True)
    loss64(f64, amp64).backward()
    g64 = amp64.grad.detach().clone()
    v = torch.as_tensor(np.random.default_rng(7).standard_normal(ny), device=dev)
    out = {}
    if fd:
        with torch.no_grad():
            one = torch.ones(ny, dtype=torch.float64, device=dev)
            lp = float(loss64(ctx64["f_0"], one + h * v))
            lm = float(loss64(ctx64["f_0"], one - h * v))
        fdv = (lp - lm) / (2 * h)
        out["fd64_directional"] = fdv
        out["grad64_rel_err_vs_fd64"] = abs(float(g64 @ v) - fdv) / abs(fdv)
    del ctx64, f64, amp64, f_t
    torch.cuda.empty_cache()

    # FP32 side: the timed forward + backward, BGK on deviations from rest (the
    # FP32 form whose sums do not cancel; XLB's BGK order is graded below)
    ctx = _build(dim, "FP32FP32", steps, collision="BGK_SHIFTED")
    c32 = _c_matrix(ctx["stepper"], torch.float32, dev)
    loss32 = _loss_fn(ctx, c32, u_target.float())

    def once():
        amp = torch.ones(ny, dtype=torch.float32, device=dev, requires_grad=True)
        f_init = ctx["f_0"].clone().requires_grad_(True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record()
        L = loss32(f_init, amp)
        e1.record()
        L.backward()
        e2.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), e1.elapsed_time(e2), amp.grad.detach().double(), f_init.grad

    once()  # warm-up
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    fwd_ms, bwd_ms, g32, gf32 = once()
    peak = torch.cuda.max_memory_allocated() - base
    cells = int(np.prod(ctx["shape"]))
    out.update({
        "workload": f"{'D2Q9' if dim == 2 else 'D3Q19'} BGK channel {'x'.join(map(str, ctx['shape']))}, 8-bump "
                    f"HalfwayBB obstacle, ZouHe parabolic inlet (peak 0.05 x per-row amplitude), ZouHe pressure "
                    f"outlet, omega 1.6, T={steps}, checkpoints every 100, loss = MSE of final velocity vs target run",
        "steps": steps,
        "cells": cells,
        "fwd_ms": fwd_ms,
        "bwd_ms": bwd_ms,
        "adjoint_to_forward": bwd_ms / fwd_ms,
        "fwd_mlups": cells * steps / (fwd_ms * 1e-3) / 1e6,
        "peak_mem_bytes": int(peak),  # above what was allocated before the timed forward
        "grad32_rel_l2_vs_grad64": float(torch.linalg.norm(g32 - g64) / torch.linalg.norm(g64)),
        "grad_f_init_finite": bool(torch.isfinite(gf32).all()),
    })
    if fd:
        out["grad32_rel_err_vs_fd64"] = abs(float(g32 @ v) - out["fd64_directional"]) / abs(out["fd64_directional"])
    del ctx
    torch.cuda.empty_cache()
    # FP32 with XLB's BGK operation order: the same adjoint, the forward summing f ~ w
    ctx = _build(dim, "FP32FP32", steps)
    loss = _loss_fn(ctx, _c_matrix(ctx["stepper"], torch.float32, dev), u_target.float())
    amp = torch.ones(ny, dtype=torch.float32, device=dev, requires_grad=True)
    loss(ctx["f_0"].clone().requires_grad_(True), amp).backward()
    gx = amp.grad.detach().double()
    out["grad32_xlb_order_rel_l2_vs_grad64"] = float(torch.linalg.norm(gx - g64) / torch.linalg.norm(g64))
    if fd:
        out["grad32_xlb_order_rel_err_vs_fd64"] = abs(float(gx @ v) - out["fd64_directional"]) / abs(
            out["fd64_directional"])
    del ctx
    torch.cuda.empty_cache()
    # FP32 store with FP64 arithmetic: separates storage rounding from arithmetic rounding
    ctx = _build(dim, "FP64FP32", steps)
    loss = _loss_fn(ctx, _c_matrix(ctx["stepper"], torch.float64, dev), u_target)
    amp = torch.ones(ny, dtype=torch.float64, device=dev, requires_grad=True)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    e0.record()
    L = loss(ctx["f_0"].clone().requires_grad_(True), amp)
    e1.record()
    L.backward()
    e2.record()
    torch.cuda.synchronize()
    out["fp64fp32_fwd_ms"] = e0.elapsed_time(e1)
    out["fp64fp32_bwd_ms"] = e1.elapsed_time(e2)
    out["grad_fp64fp32_rel_l2_vs_grad64"] = float(torch.linalg.norm(amp.grad - g64) / torch.linalg.norm(g64))
    if fd:
        out["grad_fp64fp32_rel_err_vs_fd64"] = abs(float(amp.grad @ v) - out["fd64_directional"]) / abs(
            out["fd64_directional"])
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--dim", type=int, default=2, choices=[2, 3])
    p.add_argument("--steps", type=int, default=None)
    p.add_argument("--fp32-only", action="store_true", help="FP32 forward + backward only (no FP64 checks)")
    a = p.parse_args()
    print(json.dumps(measure_fp32(a.dim, a.steps) if a.fp32_only else measure(a.dim, a.steps)))


if __name__ == "__main__":
    main()
