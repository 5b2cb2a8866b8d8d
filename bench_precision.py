"""Precision form of the lid-driven cavity: where the bytes go, and what it costs
in accuracy.

D3Q19 BGK cavity (FullwayBB on five faces, EquilibriumBC lid u = (0.05, 0, 0)),
Re = 200 with the characteristic length n - 1 (nu = 0.05 (n - 1) / 200,
omega = 1 / (3 nu + 0.5)), initial state rest equilibrium.  Populations stored
as FP32, FP16 (raw), FP16 shifted (f - w_l) and BF16 shifted, the shifted forms
also with stochastic rounding of the stores, all computed in FP32.

* Error, at 256^3 after ``--steps`` (default 10 000) steps: relative L2 of the
  velocity over the fluid cells against FP64FP64 (this library's FP64 path,
  which equals the CPU oracle bit for bit on the parity tests; the CPU oracle
  itself would need about half an hour for this run), and the mass drift
  (M(T) - M(0)) / M(0) with FP64 sums.
* Throughput, at 1024 x 1024 x 768: MLUPS of each store form over 200 steps
  after 20 warm-up steps (CUDA events).

Prints one JSON line.
"""

import argparse
import json

import torch

from bench import cavity_setup

FORMS = [("fp32", "FP32FP32"), ("fp16", "FP32FP16"), ("fp16_shifted", "FP32FP16S"), ("bf16_shifted", "FP32BF16S"),
         ("fp16_shifted_sr", "FP32FP16SR"), ("bf16_shifted_sr", "FP32BF16SR")]


def _omega(n):
    nu = 0.05 * (n - 1) / 200.0
    return 1.0 / (3.0 * nu + 0.5)


def _velocity_mass(stepper, f, bc_mask):
    """(u as float64 (3, cells) over fluid cells, total mass in float64)."""
    from xlb_gb300 import _lib

    n = stepper.grid.num_cells
    rho = torch.empty(n, dtype=torch.float64 if stepper.precision_policy.compute_code else torch.float32,
                      device=f.device)
    u = torch.empty((3, n), dtype=rho.dtype, device=f.device)
    _lib.check(stepper._lib.xlbg_macroscopic(stepper.desc, _lib.ptr(f), _lib.ptr(rho), _lib.ptr(u),
                                             _lib.stream_handle()))
    fluid = bc_mask.view(-1) == 0
    return u[:, fluid].double(), float(rho.double().sum())


def error_study(n, steps):
    out = {}
    omega = _omega(n)
    st, (f_0, f_1, bcm, mm), _ = cavity_setup(n, "FP64FP64", omega)
    m0 = _velocity_mass(st, f_0, bcm)[1]
    f_0, f_1 = st.run(f_0, f_1, bcm, mm, omega, steps)
    u_ref, m_ref = _velocity_mass(st, f_0, bcm)
    out["fp64"] = {"mass_drift": (m_ref - m0) / m0}
    del st, f_0, f_1, bcm, mm
    for name, pol in FORMS:
        st, (f_0, f_1, bcm, mm), _ = cavity_setup(n, pol, omega)
        m0 = _velocity_mass(st, f_0, bcm)[1]
        f_0, f_1 = st.run(f_0, f_1, bcm, mm, omega, steps)
        u, m = _velocity_mass(st, f_0, bcm)
        out[name] = {
            "u_rel_l2_vs_fp64": float(torch.linalg.norm(u - u_ref) / torch.linalg.norm(u_ref)),
            "mass_drift": (m - m0) / m0,
        }
        del st, f_0, f_1, bcm, mm
        torch.cuda.empty_cache()
    return out


def throughput(shape, steps=200, warmup=20):
    from bench import timed_device

    out = {}
    cells = shape[0] * shape[1] * shape[2]
    for name, pol in FORMS:
        st, fields, _ = cavity_setup(shape, pol, _omega(shape[0]))
        ms, fields = timed_device(st, fields, _omega(shape[0]), steps, warmup)
        out[name] = {"MLUPS": cells * steps / (ms * 1e-3) / 1e6}
        del st, fields
        torch.cuda.empty_cache()
    for name in out:
        out[name]["x_fp32"] = out[name]["MLUPS"] / out["fp32"]["MLUPS"]
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=256, help="cube edge of the error study")
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--big", default="1024,1024,768", help="shape of the throughput run ('' to skip)")
    a = p.parse_args()
    res = {"workload": f"D3Q19 BGK cavity, Re 200 (clength n-1), lid u=(0.05,0,0); error at {a.n}^3 after "
                       f"{a.steps} steps vs FP64FP64; throughput at {a.big}"}
    res["error"] = error_study(a.n, a.steps)
    if a.big:
        res["throughput"] = throughput(tuple(int(v) for v in a.big.split(",")))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
