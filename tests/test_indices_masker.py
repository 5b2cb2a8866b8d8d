"""Indices boundary masker kernel (``xlbg_indices_mask``) vs the oracle's masker.

Index lists with out-of-domain entries, BCs that need padding with indices in
the interior (push neighbours marked) and at the faces, BCs whose cells and
push neighbours overlap (the later BC in the list wins), a start index, 2D and
3D.  The marks are integers, so the comparison is exact.
"""

import numpy as np
import pytest

from oracle import lbm_oracle as O


def _random_bcs(rng, shape, d):
    """[(kind, indices (d, n) int64)]: a face wall, an interior blob that needs
    padding, scattered indices (some outside the domain), a velocity inlet."""
    grids = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    wall = np.array([g[(grids[1] == 0)] for g in grids])
    center = [s // 2 for s in shape]
    r2 = sum((g - c) ** 2 for g, c in zip(grids, center))
    blob = np.array([g[r2 < (min(shape) // 4) ** 2] for g in grids])
    n = 40
    scattered = np.stack([rng.integers(-2, s + 2, size=n) for s in shape])
    keep = np.ones(n, dtype=bool)
    for k in range(n):  # no repeats inside one BC (XLB's overlap check rejects them)
        keep[k] = not any(np.array_equal(scattered[:, k], scattered[:, j]) for j in range(k) if keep[j])
    scattered = scattered[:, keep]
    inlet = np.array([g[(grids[0] == shape[0] - 1) & (grids[1] > 0)] for g in grids])
    return [("fullway_bb", wall), ("halfway_bb", blob), ("halfway_bb", scattered), ("equilibrium", inlet)]


def _xlb_bc(kind, idx):
    from xlb_gb300.operator import boundary_condition as B

    if kind == "fullway_bb":
        return B.FullwayBounceBackBC(indices=idx.tolist())
    if kind == "halfway_bb":
        return B.HalfwayBounceBackBC(indices=idx.tolist())
    u = (0.02,) + (0.0,) * (idx.shape[0] - 1)
    return B.EquilibriumBC(rho=1.0, u=u, indices=idx.tolist())


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape", [("D2Q9", (23, 17)), ("D3Q19", (15, 12, 10)), ("D3Q27", (13, 11, 9))])
def test_indices_masker_matches_oracle(lattice, shape):
    import torch

    import xlb_gb300 as xlb
    from xlb_gb300.operator.boundary_masker import IndicesBoundaryMasker

    pp = xlb.PrecisionPolicy.FP32FP32
    vs = getattr(xlb.velocity_set, lattice)(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    d = len(shape)
    lat = O.Lattice(lattice)
    spec = _random_bcs(np.random.default_rng(3), shape, d)
    xbcs = [_xlb_bc(k, idx) for k, idx in spec]
    obcs = [O.BC(k, bc.id, idx) for (k, idx), bc in zip(spec, xbcs)]
    want_bm, want_mm = O.masker(lat, shape, obcs)
    s3 = shape if d == 3 else shape + (1,)
    bm = torch.zeros((1,) + s3, dtype=torch.uint8, device="cuda")
    mm = torch.zeros((lat.q,) + s3, dtype=torch.bool, device="cuda")
    bm, mm = IndicesBoundaryMasker(vs, pp)(xbcs, bm, mm)
    torch.cuda.synchronize()
    assert np.array_equal(bm.cpu().numpy(), want_bm)
    assert np.array_equal(mm.cpu().numpy(), want_mm)
    # the layouts exercise what they are meant to: push marks, and cells of an
    # earlier BC taken over by a later one
    alone, _ = O.masker(lat, shape, obcs[:2])
    assert (alone == xbcs[1].id).sum() > spec[1][1].shape[1]
    assert ((alone == xbcs[1].id) & (want_bm != xbcs[1].id)).sum() > 0
    assert (want_bm == xbcs[3].id).sum() > 0


@pytest.mark.gpu
def test_indices_masker_start_index_and_prior_marks():
    import torch

    import xlb_gb300 as xlb
    from xlb_gb300.operator.boundary_masker import IndicesBoundaryMasker

    pp = xlb.PrecisionPolicy.FP32FP32
    vs = xlb.velocity_set.D3Q19(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    shape = (12, 10, 9)
    lat = O.Lattice("D3Q19")
    start = np.array([5, -2, 3])
    spec = _random_bcs(np.random.default_rng(8), shape, 3)
    xbcs = [_xlb_bc(k, idx + start[:, None]) for k, idx in spec]  # global indices
    obcs = [O.BC(k, bc.id, idx) for (k, idx), bc in zip(spec, xbcs)]  # local indices
    want_bm, want_mm = O.masker(lat, shape, obcs)
    rng = np.random.default_rng(1)
    prior_bm = np.where(rng.random((1,) + shape) < 0.1, 77, 0).astype(np.uint8)
    prior_mm = rng.random((lat.q,) + shape) < 0.05
    touched = (want_bm != 0)
    want_bm = np.where(touched, want_bm, prior_bm)
    want_mm = want_mm | prior_mm
    bm = torch.from_numpy(prior_bm).cuda()
    mm = torch.from_numpy(prior_mm).cuda()
    bm, mm = IndicesBoundaryMasker(vs, pp)(xbcs, bm, mm, start_index=start)
    torch.cuda.synchronize()
    assert np.array_equal(bm.cpu().numpy(), want_bm)
    assert np.array_equal(mm.cpu().numpy(), want_mm)


@pytest.mark.gpu
def test_stepper_repacks_after_masker_writes():
    """The stepper caches the packed missing bits against the mask tensors.  The
    maskers write the masks through raw pointers, which torch does not see, so
    they bump the tensors' version counters: a step after re-masking must use
    the new marks, and another mask tensor (even one at a reused address) must
    never hit the cache."""
    import torch

    import xlb_gb300 as xlb
    from _scenarios import Scenario
    from xlb_gb300.operator.boundary_condition import HalfwayBounceBackBC
    from xlb_gb300.operator.boundary_masker import IndicesBoundaryMasker

    sc = Scenario("D3Q19", (16, 12, 12), "channel_zouhe", policy="fp32")
    f_0, f_1, bcm, mm = sc.gpu_fields()
    f_0, f_1 = sc.stepper(f_0, f_1, bcm, mm, sc.omega, 0)
    bits0 = sc.stepper._aux_state(bcm, mm)[0]
    before = bits0.clone()

    g = np.meshgrid(*[np.arange(s) for s in (16, 12, 12)], indexing="ij")
    block = (g[0] >= 6) & (g[0] < 9) & (g[1] >= 4) & (g[1] < 7) & (g[2] >= 4) & (g[2] < 7)
    idx = np.array([a[block] for a in g])
    pp = xlb.PrecisionPolicy.FP32FP32
    IndicesBoundaryMasker(xlb.velocity_set.D3Q19(pp), pp)([HalfwayBounceBackBC(indices=idx.tolist())], bcm, mm)
    bits1 = sc.stepper._aux_state(bcm, mm)[0]
    m = mm.cpu().numpy().reshape(19, -1).astype(np.int64)
    want = np.bitwise_or.reduce(m << np.arange(19)[:, None], axis=0)
    assert np.array_equal(bits1.cpu().numpy().astype(np.int64) & 0x7FFFF, want)
    assert not torch.equal(bits1, before)

    # a different mask tensor with other contents is packed afresh
    mm2 = torch.zeros_like(mm)
    bits2 = sc.stepper._aux_state(bcm, mm2)[0]
    assert int(bits2.abs().sum()) == 0
