"""The oracle against golden vectors produced by XLB's own stepper source.

tests/golden/make_golden.py ran XLB's Warp code path (FP64FP64) unmodified under a
CPU emulation of the Warp API and stored, per case: XLB's masker output, its
prepare_fields() populations (equilibrium init + ZouHe/Regularized aux data), a
perturbed input state, the state after a few steps, and, in 3D, XLB's
MomentumTransfer force on the final state.  Every piece is replayed here
through the oracle.
"""

import glob
import os

import numpy as np
import pytest

from oracle import lbm_oracle as O

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz"))
          if not os.path.basename(p).startswith(("mesh_", "render_")))  # those: test_mesh_masker.py, test_renderer.py


def load(path):
    g = dict(np.load(path, allow_pickle=False))
    lat = O.Lattice(str(g["lattice"]))
    table = g["profile_table"]

    def profile(idx3):
        return 0.04 * (1.0 + table[idx3[1], idx3[2]])

    bcs = []
    for k, (bid, kind, val, u) in enumerate(zip(g["bc_ids"], g["bc_kinds"], g["bc_values"], g["bc_u"])):
        kind = str(kind)
        bcs.append(O.BC(kind, int(bid), g[f"bc{k}_indices"], rho=float(val) if kind == "equilibrium" else 1.0,
                        u=tuple(u), value=None if np.isnan(val) else float(val),
                        profile=profile if np.isnan(val) else None))
    return g, lat, bcs


def test_fixtures_present():
    assert len(GOLDEN) >= 8


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_masker_matches_xlb(path):
    g, lat, bcs = load(path)
    bcm, miss = O.masker(lat, tuple(int(s) for s in g["shape"]), bcs)
    assert np.array_equal(bcm, g["bc_mask"])
    assert np.array_equal(miss, g["missing_mask"])


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_prepare_fields_matches_xlb(path):
    g, lat, bcs = load(path)
    st = O.Store("f64", lat)
    shape = tuple(int(s) for s in g["shape"])
    f0 = O.initial_equilibrium(lat, st, shape, np.float64)
    assert np.array_equal(f0, g["prep_f0"])
    f1 = O.aux_init(lat, st, f0.copy(), g["bc_mask"], g["missing_mask"], bcs, np.float64)
    assert np.array_equal(f1, g["prep_f1"])


def _run(g, lat, bcs, recovery):
    st = O.Store("f64", lat)
    with np.errstate(all="ignore"):
        return O.run(lat, st, g["in_f0"].copy(), g["in_f1"].copy(), g["bc_mask"], g["missing_mask"], float(g["omega"]),
                     bcs, int(g["steps"]), str(g["collision"]), np.float64, recovery=recovery)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_steps_match_xlb(path):
    """XLB's source run sequentially in cell order resolves its aux-recovery race
    as recovery-before-read for these layouts (inlet at x = 0): the oracle in that
    order matches it everywhere to 1e-14."""
    g, lat, bcs = load(path)
    a, b = _run(g, lat, bcs, "before")
    for got, want, name in ((a, g["out_f0"], "f_0"), (b, g["out_f1"], "f_1")):
        err = np.max(np.abs(got - want))
        assert err <= 1e-14, f"{name}: max |oracle - XLB| = {err:.3e}"


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_steps_match_xlb_outside_the_race(path):
    """The order the CUDA path uses (recovery after every read) matches XLB
    wherever the two orders agree; where they differ, only boundary cells that
    bounce a value pulled through the periodic wrap from an aux-recovery slot are
    involved, never fluid cells."""
    g, lat, bcs = load(path)
    a, b = _run(g, lat, bcs, "after")
    a2, b2 = _run(g, lat, bcs, "before")
    for got, alt, want, name in ((a, a2, g["out_f0"], "f_0"), (b, b2, g["out_f1"], "f_1")):
        same = got == alt
        err = np.max(np.abs(got - want)[same])
        assert err <= 1e-14, f"{name}: max |oracle - XLB| outside the race = {err:.3e}"
        raced = np.argwhere(~same)
        ids = {int(g["bc_mask"][(0,) + tuple(r[1:])]) for r in raced}
        assert 0 not in ids, "a fluid cell depends on the recovery order"


@pytest.mark.parametrize("path", [p for p in GOLDEN if "force" in np.load(p).files],
                         ids=[os.path.basename(p)[:-4] for p in GOLDEN if "force" in np.load(p).files])
def test_momentum_transfer_matches_xlb(path):
    g, lat, bcs = load(path)
    st = O.Store("f64", lat)
    force = O.momentum_transfer(lat, st, g["out_f0"], g["bc_mask"], g["missing_mask"], int(g["force_bc_id"]), np.float64)
    assert np.allclose(force, g["force"], rtol=1e-12, atol=1e-13)


_KIND = {"fullway_bb": 1, "halfway_bb": 2, "equilibrium": 3, "zouhe_velocity": 4, "zouhe_pressure": 5,
         "regularized_velocity": 6, "regularized_pressure": 7, "extrapolation": 8}


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_cuda_path_matches_xlb(path):
    """The CUDA path, called through the C ABI in FP64, on XLB's own inputs: equal
    to the oracle's recovery-after order, and to XLB's output outside the race."""
    import torch

    from xlb_gb300 import _lib

    g, lat, bcs = load(path)
    lib = _lib.load()
    shape = tuple(int(s) for s in g["shape"])
    d = _lib.Desc()
    d.abi_version, d.lattice, d.store, d.compute = _lib.ABI_VERSION, {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}[lat.name], 1, 1
    d.collision = 1 if str(g["collision"]) == "KBC" else 0
    d.nx, d.ny, d.nz = shape if len(shape) == 3 else shape + (1,)
    d.nbc = len(bcs)
    for i, bc in enumerate(bcs):
        d.bc[i].id, d.bc[i].kind, d.bc[i].rho = bc.id, _KIND[bc.kind], float(bc.rho)
        for k in range(3):
            d.bc[i].u[k] = float(bc.u[k])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    f0, f1 = dev(g["in_f0"]), dev(g["in_f1"])
    bcm, mm = dev(g["bc_mask"]), dev(g["missing_mask"])
    bits = torch.empty(bcm.numel(), dtype=torch.int32, device="cuda")
    s = _lib.stream_handle()
    P = _lib.ptr
    _lib.check(lib.xlbg_pack_missing(d, P(mm), P(bits), s))
    rec_ids = torch.tensor([bc.id for bc in bcs if bc.kind in O.RECOVERY_KINDS] or [0], dtype=torch.uint8, device="cuda")
    rec = torch.nonzero(torch.isin(bcm.view(-1), rec_ids)).view(-1).to(torch.int64).contiguous()
    scratch = torch.empty(max(1, rec.numel()) * lat.q, dtype=torch.float64, device="cuda")
    nrec = rec.numel() if len(rec_ids) and any(bc.kind in O.RECOVERY_KINDS for bc in bcs) else 0
    for t in range(int(g["steps"])):
        _lib.check(lib.xlbg_step(d, P(f0), P(f1), P(bcm), P(bits), P(rec) if nrec else None, nrec,
                                 P(scratch) if nrec else None, float(g["omega"]), t, s))
        f0, f1 = f1, f0
    torch.cuda.synchronize()
    a, b = f0.cpu().numpy(), f1.cpu().numpy()
    want_a, want_b = _run(g, lat, bcs, "after")
    alt_a, alt_b = _run(g, lat, bcs, "before")
    assert np.array_equal(a, want_a) and np.array_equal(b, want_b)
    for got, alt, ref in ((a, alt_a, g["out_f0"]), (b, alt_b, g["out_f1"])):
        same = want_a.shape == got.shape and (alt == got)
        assert np.max(np.abs(got - ref)[same]) <= 1e-14
