"""Macroscopic read-out (``xlbg_macroscopic``, xlb/operator/macroscopic/macroscopic.py:39-66)
against the oracle's macroscopic (zero_moment.py:22-27, first_moment.py:25-38) on
perturbed states, for every store form.  The kernel decodes as the step does and
keeps XLB's summation order, so rho and u match bit for bit."""

import numpy as np
import pytest

from oracle import lbm_oracle as O
from _scenarios import Scenario


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64", "f16", "f16s", "bf16s", "fp64f32", "fp64f16"])
@pytest.mark.parametrize("lattice,shape", [("D2Q9", (30, 18)), ("D3Q19", (12, 10, 9)), ("D3Q27", (10, 8, 16))])
def test_macroscopic_matches_oracle(lattice, shape, policy):
    import torch

    from xlb_gb300.operator.macroscopic import Macroscopic

    sc = Scenario(lattice, shape, "periodic", policy=policy)
    sc.randomize(seed=51, amp=0.2)
    f = sc.to_torch(sc.f0)
    rho, u = Macroscopic()(f)
    torch.cuda.synchronize()
    want_rho, want_u = O.macroscopic(sc.lat, sc.store.decode(sc.f0, sc.T), sc.T)
    assert np.array_equal(rho.cpu().numpy()[0], want_rho)
    assert np.array_equal(u.cpu().numpy(), np.stack(want_u))


@pytest.mark.gpu
def test_macroscopic_after_steps_and_caller_buffers():
    """After a few steps of a channel, into caller-provided rho / u buffers."""
    import torch

    from xlb_gb300.operator.macroscopic import Macroscopic

    sc = Scenario("D3Q19", (16, 10, 10), "channel_regularized", policy="fp32")
    sc.randomize(seed=52)
    got0, _ = sc.gpu_steps(3)
    want0, _ = sc.oracle_steps(3)
    f = sc.to_torch(got0)
    rho = torch.full((1,) + f.shape[1:], float("nan"), dtype=torch.float32, device="cuda")
    u = torch.full((3,) + f.shape[1:], float("nan"), dtype=torch.float32, device="cuda")
    r2, u2 = Macroscopic()(f, rho, u)
    assert r2 is rho and u2 is u
    want_rho, want_u = O.macroscopic(sc.lat, sc.store.decode(want0, sc.T), sc.T)
    assert np.array_equal(rho.cpu().numpy()[0], want_rho)
    assert np.array_equal(u.cpu().numpy(), np.stack(want_u))
