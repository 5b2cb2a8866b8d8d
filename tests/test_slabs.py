"""Slab decomposition along x (XLB's distribute.py:10-105 / parallel_operator.py:6-82).

CPU (no GPU): the slab layout; the ghost-plane schedule with every slab
stepped by the oracle, in one process (LocalTransport) and over two gloo ranks
(ProcessGroupTransport), against the single-domain oracle run, bit for bit; the
FP64 all-reduce of the diagnostics.

GPU: two and three slabs on one GPU (device-local ghost copies) against the
single-domain CUDA step for every boundary layout, bit for bit, and the fused
FP64 mass / force summed over slabs against the single-domain diagnostics step.
"""

import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import lbm_oracle as O
from _scenarios import Scenario

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))

LAYOUTS = [
    ("D3Q19", (15, 8, 8), "cavity_fullway"),
    ("D3Q19", (15, 8, 8), "cavity_halfway"),
    ("D3Q19", (16, 10, 10), "channel_zouhe"),
    ("D3Q19", (16, 10, 10), "channel_regularized"),
    ("D3Q19", (14, 9, 8), "channel_pressure"),
    ("D3Q27", (13, 8, 8), "channel_regularized"),
    ("D2Q9", (30, 18), "channel_zouhe"),
    ("D2Q9", (24, 20), "periodic"),
]


def test_slab_layout():
    from xlb_gb300.distribute import SlabLayout

    lay = SlabLayout(10, 3)
    assert lay.bounds == [(0, 4), (4, 7), (7, 10)]
    assert lay.padded_planes(0) == [9, 0, 1, 2, 3, 4]
    assert lay.padded_planes(2) == [6, 7, 8, 9, 0]
    with pytest.raises(ValueError):
        SlabLayout(4, 5)


def test_crossing_sets_match_velocity_set():
    import xlb_gb300 as xlb
    from xlb_gb300.distribute import crossing_directions

    pp = xlb.PrecisionPolicy.FP32FP32
    for cls, q, k in ((xlb.velocity_set.D2Q9, 9, 3), (xlb.velocity_set.D3Q19, 19, 5), (xlb.velocity_set.D3Q27, 27, 9)):
        vs = cls(pp)
        right, left = crossing_directions(vs)
        assert len(right) == len(left) == k
        assert all(vs.c[0, l] == 1 for l in right) and all(vs.c[0, l] == -1 for l in left)


def _oracle_local_step(sc):
    """A per-slab step by the oracle on CPU tensors (what the CUDA step does on a slab)."""

    def step(s, omega, timestep):
        f0, f1 = s.f_0.numpy(), s.f_1.numpy()
        with np.errstate(all="ignore"):
            n0, n1 = O.step(sc.lat, sc.store, f0, f1, s.bc_mask.numpy(), s.missing_mask.numpy(), omega, sc.obcs,
                            sc.collision, sc.T)
        s.f_0.copy_(torch.from_numpy(n0))
        s.f_1.copy_(torch.from_numpy(n1))

    return step


def _cpu_fields(sc):
    return (torch.from_numpy(sc.f0.copy()), torch.from_numpy(sc.f1.copy()), torch.from_numpy(sc.bc_mask.copy()),
            torch.from_numpy(sc.missing.copy()))


@pytest.mark.parametrize("n_slabs", [2, 3])
@pytest.mark.parametrize("lattice,shape,layout", LAYOUTS[2:4] + LAYOUTS[6:7])
def test_local_schedule_with_oracle_steps(lattice, shape, layout, n_slabs):
    from xlb_gb300.distribute import DistributedStepper, LocalTransport

    sc = Scenario(lattice, shape, layout, policy="fp32")
    sc.randomize(seed=61)
    want0, want1 = sc.oracle_steps(3)
    ds = DistributedStepper(sc.stepper, n_slabs=n_slabs, transport=LocalTransport(), local_step=_oracle_local_step(sc))
    slabs = ds.scatter(*_cpu_fields(sc))
    ds.run(slabs, sc.omega, 3)
    got0, got1 = ds.gather(slabs)
    assert np.array_equal(got0.numpy(), want0) and np.array_equal(got1.numpy(), want1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, spec, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    from xlb_gb300.distribute import DistributedStepper, ProcessGroupTransport

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lattice, shape, layout = spec
        sc = Scenario(lattice, shape, layout, policy="fp64")
        sc.randomize(seed=62)
        ds = DistributedStepper(sc.stepper, transport=ProcessGroupTransport(), local_step=_oracle_local_step(sc))
        assert ds.layout.n == world and ds.local == [rank]
        (s,) = ds.scatter(*_cpu_fields(sc))
        ds.run([s], sc.omega, 3)
        out[rank] = (s.x0, s.x1, s.f_0[:, 1 : s.t + 1].numpy().copy(), s.f_1[:, 1 : s.t + 1].numpy().copy())
        # the FP64 all-reduce the diagnostics use
        t = torch.tensor([float(rank + 1), 0.5, -1.0, 2.0 ** -40], dtype=torch.float64)
        red = ds.transport.all_reduce(t)
        out[("sum", rank)] = red.numpy().copy()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("lattice,shape,layout", [LAYOUTS[3], LAYOUTS[6]])
def test_two_gloo_ranks_match_single_domain(lattice, shape, layout):
    sc = Scenario(lattice, shape, layout, policy="fp64")
    sc.randomize(seed=62)
    want0, want1 = sc.oracle_steps(3)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_gloo_rank, args=(2, _free_port(), (lattice, shape, layout), out), nprocs=2, join=True,
                           start_method="spawn")
        res = dict(out)
    parts = sorted((res[r] for r in (0, 1)), key=lambda p: p[0])
    got0 = np.concatenate([p[2] for p in parts], axis=1)
    got1 = np.concatenate([p[3] for p in parts], axis=1)
    assert parts[0][0] == 0 and parts[-1][1] == shape[0]
    assert np.array_equal(got0, want0) and np.array_equal(got1, want1)
    for r in (0, 1):
        assert np.array_equal(res[("sum", r)], np.array([3.0, 1.0, -2.0, 2.0 ** -39]))


@pytest.mark.gpu
@pytest.mark.parametrize("n_slabs", [2, 3])
@pytest.mark.parametrize("policy", ["fp32", "f16s"])
@pytest.mark.parametrize("lattice,shape,layout", LAYOUTS)
def test_slabs_on_one_gpu_match_single_domain(lattice, shape, layout, policy, n_slabs):
    from xlb_gb300.distribute import DistributedStepper, LocalTransport

    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=63)
    want0, want1 = sc.gpu_steps(4)
    ds = DistributedStepper(sc.stepper, n_slabs=n_slabs, transport=LocalTransport())
    slabs = ds.scatter(*sc.gpu_fields())
    ds.run(slabs, sc.omega, 4)
    got0, got1 = ds.gather(slabs)
    torch.cuda.synchronize()
    assert np.array_equal(sc.to_numpy(got0), want0) and np.array_equal(sc.to_numpy(got1), want1)


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,layout,force_idx", [("D3Q19", (16, 10, 10), "channel_regularized", 3),
                                                            ("D2Q9", (30, 18), "channel_zouhe", 3)])
def test_slab_diagnostics_match_single_domain(lattice, shape, layout, force_idx):
    """Mass and momentum-exchange force summed in FP64 per slab and over slabs
    equal the single-domain diagnostics step's (the cross-cell FP64 order
    differs: rtol 1e-12)."""
    from xlb_gb300.distribute import DistributedStepper, LocalTransport

    sc = Scenario(lattice, shape, layout, policy="fp32")
    sc.randomize(seed=64)
    f_0, f_1, bcm, mm = sc.gpu_fields()
    force_bc = sc.xbcs[force_idx]
    ds = DistributedStepper(sc.stepper, n_slabs=2, transport=LocalTransport())
    slabs = ds.scatter(f_0, f_1, bcm, mm)
    for t in range(3):
        f_0, f_1, want = sc.stepper.step_with_diagnostics(f_0, f_1, bcm, mm, sc.omega, t, force_bc=force_bc)
        f_0, f_1 = f_1, f_0
        got = ds.step_with_diagnostics(slabs, sc.omega, t, force_bc=force_bc)
        assert np.allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-12, atol=1e-12)
    g0, _ = ds.gather(slabs)
    assert torch.equal(g0, f_0)


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,layout", [("D3Q19", (16, 10, 10), "channel_regularized"),
                                                  ("D3Q19", (15, 8, 8), "cavity_fullway"),
                                                  ("D2Q9", (30, 18), "channel_zouhe")])
def test_slab_prepare_fields_equals_scattered_global(lattice, shape, layout):
    """prepare_fields() per slab (global masks, slab populations and aux values
    only) gives the slabs that scattering the global prepare_fields() gives."""
    from xlb_gb300.distribute import DistributedStepper, LocalTransport

    sc = Scenario(lattice, shape, layout, policy="fp32")
    ds = DistributedStepper(sc.stepper, n_slabs=3, transport=LocalTransport())
    a = ds.scatter(*sc.stepper.prepare_fields())
    for bc in sc.xbcs:
        bc.is_initialized_with_aux_data = False
    b = ds.prepare_fields()
    for sa, sb in zip(a, b):
        for name in ("bc_mask", "missing_mask"):
            assert torch.equal(getattr(sa, name), getattr(sb, name)), (sa.index, name)
        # populations of the interior planes (ghost planes are refilled before every
        # step, and a ghost cell's f_1 is never read)
        for name in ("f_0", "f_1"):
            assert torch.equal(getattr(sa, name)[:, 1 : sa.t + 1], getattr(sb, name)[:, 1 : sb.t + 1]), (sa.index, name)
