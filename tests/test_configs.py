"""Workload-size checks.

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
