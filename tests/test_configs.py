"""Workload-size checks: C1 at full size, C3 at a reduced size.

C1: the 2D lid-driven cavity at its full size -- D2Q9 BGK 256 x 256, FullwayBB on
the left, right and bottom walls, EquilibriumBC lid (rho 1, u = (0.05, 0)) on the
top face without edges, Re 200 (nu = 0.05 * 255 / 200, omega = 1 / (3 nu + 0.5)),
rest-equilibrium start, 5000 steps -- against the C restatement of the step in
FP64 (the oracle; gcc without FMA contraction, equal to the numpy oracle bit for
bit).  The FP64 GPU path must match it exactly; the FP32 GPU path must match its
velocity to 1e-3 relative L2 (measured 2.8e-4: FP32 rounding accumulated over
5000 steps), its density to 1e-4 (measured 8.3e-6) and its total mass to 1e-4.
"""

import numpy as np
import pytest

from _scenarios import Scenario
from oracle import cref

C1_OMEGA = 1.0 / (3.0 * (0.05 * 255 / 200) + 0.5)
C1_STEPS = 5000


def _rho_u(lat, f):
    f = f.astype(np.float64).reshape(lat.q, -1)
    rho = f.sum(0)
    u = (lat.c.astype(np.float64) @ f) / rho
    return rho, u


@pytest.fixture(scope="module")
def c1_oracle():
    sc = Scenario("D2Q9", (256, 256), "cavity_fullway", "fp64", "BGK", omega=C1_OMEGA)
    st = cref.Stepper(sc.lat, sc.shape, sc.bc_mask, sc.missing, sc.obcs, "BGK", np.float64, threads=0)
    f_new, _ = st.run(sc.f0.copy(), sc.f1.copy(), C1_OMEGA, C1_STEPS)
    return sc, f_new


@pytest.mark.gpu
def test_c1_fp64_equals_oracle(c1_oracle):
    sc_o, want = c1_oracle
    sc = Scenario("D2Q9", (256, 256), "cavity_fullway", "fp64", "BGK", omega=C1_OMEGA)
    got, _ = sc.gpu_steps(C1_STEPS, use_run=True)
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_c1_fp32_close_to_fp64_oracle(c1_oracle):
    sc_o, want = c1_oracle
    sc = Scenario("D2Q9", (256, 256), "cavity_fullway", "fp32", "BGK", omega=C1_OMEGA)
    got, _ = sc.gpu_steps(C1_STEPS, use_run=True)
    rho_w, u_w = _rho_u(sc_o.lat, want)
    rho_g, u_g = _rho_u(sc.lat, got)
    err_u = np.linalg.norm(u_g - u_w) / np.linalg.norm(u_w)
    err_rho = np.linalg.norm(rho_g - rho_w) / np.linalg.norm(rho_w)
    # the lid's EquilibriumBC does not conserve mass, so FP32 mass is compared with the oracle's
    m_w = float(want.astype(np.float64).sum())
    err_m = abs(float(got.astype(np.float64).sum()) - m_w) / m_w
    msg = f"u {err_u:.3e} rho {err_rho:.3e} mass {err_m:.3e}"
    assert err_u < 1e-3, msg
    assert err_rho < 1e-4, msg
    assert err_m < 1e-4, msg


# C3 reduced: the sphere-channel layout of the D3Q27 KBC external-flow workload
# (FullwayBB side walls, Regularized velocity inlet 0.04 +-1 % per cell,
# ExtrapolationOutflow, HalfwayBB sphere) on 192 x 48 x 48 cells with the
# workload's omega (Re 1000 on a 48-cell sphere: nu = 0.04 * 48 / 1000).
C3R_SHAPE = (192, 48, 48)
C3R_OMEGA = 1.0 / (3.0 * (0.04 * 48 / 1000.0) + 0.5)


@pytest.fixture(scope="module")
def c3r_oracles():
    out = {}
    for policy, T in (("fp32", np.float32), ("fp64", np.float64)):
        sc = Scenario("D3Q27", C3R_SHAPE, "channel_regularized", policy, "KBC", omega=C3R_OMEGA)
        st = cref.Stepper(sc.lat, sc.shape, sc.bc_mask, sc.missing, sc.obcs, "KBC", T, threads=0)
        out[policy] = st.run(sc.f0.copy(), sc.f1.copy(), C3R_OMEGA, 200)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64"])
def test_c3_reduced_equals_c_oracle(c3r_oracles, policy):
    """200 steps of the reduced sphere channel (FP32: the TMA-staged KBC kernel;
    FP64: the marching kernel) equal the C restatement bit for bit."""
    want0, want1 = c3r_oracles[policy]
    sc = Scenario("D3Q27", C3R_SHAPE, "channel_regularized", policy, "KBC", omega=C3R_OMEGA)
    got0, got1 = sc.gpu_steps(200, use_run=True)
    np.testing.assert_array_equal(got0, want0)
    np.testing.assert_array_equal(got1, want1)


@pytest.mark.gpu
def test_c3_reduced_fp32_close_to_fp64():
    """FP32 against FP64 after 100 steps of the reduced sphere channel (the FP64
    path equals the oracle bit for bit, above): velocity 5e-5 and density 5e-6
    relative L2 over the fluid cells, force (MomentumTransfer on the sphere) 1e-4
    of the drag.  Measured with the C restatement, which both GPU paths equal:
    u 1.3e-5, rho 1.0e-6, force 2.1e-5 at 100 steps.  The FP32 and FP64 runs then
    part quickly in this impulsively started, under-resolved KBC flow (omega
    1.977): u 1.0e-4 / 2.8e-4 / 9.5e-4 and force 1 % / 2.3 % / 4.1 % at 200 /
    300 / 500 steps."""
    from xlb_gb300.operator.force import MomentumTransfer

    res = {}
    for policy in ("fp64", "fp32"):
        sc = Scenario("D3Q27", C3R_SHAPE, "channel_regularized", policy, "KBC", omega=C3R_OMEGA)
        f_0, f_1, bcm, mm = sc.gpu_fields()
        f_0, f_1 = sc.stepper.run(f_0, f_1, bcm, mm, sc.omega, 100)
        force = MomentumTransfer(sc.xbcs[3])(f_0, f_1, bcm, mm)
        rho, u = _rho_u(sc.lat, sc.to_numpy(f_0))
        fluid = sc.bc_mask.reshape(-1) == 0
        res[policy] = (rho[fluid], u[:, fluid], force)
    (r64, u64, F64), (r32, u32, F32) = res["fp64"], res["fp32"]
    err_u = np.linalg.norm(u32 - u64) / np.linalg.norm(u64)
    err_rho = np.linalg.norm(r32 - r64) / np.linalg.norm(r64)
    err_f = np.max(np.abs(F32 - F64)) / abs(F64[0])
    msg = f"u {err_u:.3e} rho {err_rho:.3e} force {err_f:.3e} (F64 {F64}, F32 {F32})"
    assert np.all(np.isfinite(u32)) and abs(F64[0]) > 0, msg
    assert err_u < 5e-5 and err_rho < 5e-6 and err_f < 1e-4, msg
