"""Fused FP64 diagnostics (mass of the new state, momentum-exchange force on the
input state) against the oracle's total_mass / momentum_transfer
(xlb/operator/force/momentum_transfer.py:92-176).  Per-cell sums are in the
compute type as in XLB; only the cross-cell FP64 summation order differs, so
rtol = 1e-12."""

import numpy as np
import pytest

from oracle import lbm_oracle as O
from _scenarios import Scenario


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64", "bf16s", "f16s", "f16sr", "bf16sr"])
@pytest.mark.parametrize(
    "lattice,shape,layout,collision,force_idx",
    [
        ("D3Q19", (16, 10, 10), "channel_regularized", "BGK", 3),
        ("D2Q9", (30, 18), "channel_zouhe", "BGK", 3),
        ("D3Q27", (16, 10, 10), "channel_regularized", "KBC", 3),
        ("D3Q19", (12, 10, 9), "cavity_halfway", "BGK", 1),
        # FP32 D3Q27 KBC on a contiguous axis of 16: the TMA-staged diagnostics step
        ("D3Q27", (16, 10, 16), "channel_regularized", "KBC", 3),
        # shifted 16-bit stores on contiguous axes of multiples of 8: the segmented
        # kernel's diagnostics step (one segment; segments of 256 and 8)
        ("D3Q19", (16, 10, 16), "channel_zouhe", "BGK", 3),
        ("D3Q19", (6, 5, 264), "cavity_halfway", "BGK", 1),
    ],
)
def test_diagnostics_match_oracle(lattice, shape, layout, collision, force_idx, policy):
    import torch

    if collision == "KBC" and policy.endswith("sr"):
        pytest.skip("stochastic rounding is a store of BGK on deviations")

    sc = Scenario(lattice, shape, layout, policy=policy, collision=collision)
    sc.randomize(seed=31)
    f_0, f_1, bcm, mm = sc.gpu_fields()
    force_bc = sc.xbcs[force_idx]
    f0_np, f1_np = sc.f0.copy(), sc.f1.copy()
    for t in range(3):
        # oracle: force on the input state, mass of the output state
        want_force = O.momentum_transfer(sc.lat, sc.store, f0_np, sc.bc_mask, sc.missing, force_bc.id, sc.T)
        with np.errstate(all="ignore"):
            n0, n1 = O.step(sc.lat, sc.store, f0_np, f1_np, sc.bc_mask, sc.missing, sc.omega, sc.obcs, sc.collision, sc.T,
                            timestep=t)
        want_mass = O.total_mass(sc.lat, sc.store, n1, sc.bc_mask, sc.T)
        f_0, f_1, out = sc.stepper.step_with_diagnostics(f_0, f_1, bcm, mm, sc.omega, t, force_bc=force_bc)
        got = out.cpu().numpy()
        assert np.isclose(got[0], want_mass, rtol=1e-12, atol=0), (t, got[0], want_mass)
        assert np.allclose(got[1 : 1 + sc.lat.d], want_force, rtol=1e-12, atol=1e-10), (t, got, want_force)
        assert np.array_equal(sc.to_numpy(f_1), n1)
        f0_np, f1_np = n1, n0
        f_0, f_1 = f_1, f_0
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_mass_without_force():
    sc = Scenario("D2Q9", (24, 20), "cavity_fullway", policy="fp64")
    sc.randomize(seed=32)
    f_0, f_1, bcm, mm = sc.gpu_fields()
    f_0, f_1, out = sc.stepper.step_with_diagnostics(f_0, f_1, bcm, mm, sc.omega, 0)
    _, n1 = O.step(sc.lat, sc.store, sc.f0, sc.f1, sc.bc_mask, sc.missing, sc.omega, sc.obcs, "BGK", sc.T)
    got = out.cpu().numpy()
    assert np.isclose(got[0], O.total_mass(sc.lat, sc.store, n1, sc.bc_mask, sc.T), rtol=1e-12)
    assert np.all(got[1:] == 0.0)
