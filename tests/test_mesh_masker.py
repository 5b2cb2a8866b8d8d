"""Mesh boundary masker: oracle vs XLB's own masker (golden vectors), CUDA
kernels vs the oracle, and the stepper with a mesh BC.

The golden files tests/golden/mesh_*.npz come from XLB's MeshBoundaryMasker
source run under the CPU Warp emulator (tests/golden/make_golden_mesh.py), with
Warp's copy semantics for nested subscript stores (``bc_mask``) and with
element stores that write (``bc_mask_edges``).  Voxel tests and marks are
integer results of float32 arithmetic done in the same order everywhere, so
every comparison is exact.
"""

import os

import numpy as np
import pytest

from oracle import lbm_oracle as O
from oracle import mesh_oracle as M

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = ["d3q19", "d3q27"]


def _golden(name):
    return np.load(os.path.join(HERE, "golden", f"mesh_{name}.npz"))


def _meshes(g, edges):
    key = "_id_edges" if edges else "_id"
    return [(g[f"mesh{k}_vertices"], int(g[f"mesh{k}{key}"])) for k in range(int(g["n_mesh"]))]


def _oracle_apply(lat, shape, meshes, bc_mask, missing, edges):
    for verts, bid in meshes:
        M.mask(lat, shape, np.asarray(verts, dtype=np.float32).reshape(-1, 3, 3), bid, bc_mask, missing, edges)
    return bc_mask, missing


@pytest.mark.parametrize("edges", [False, True])
@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_xlb_masker(name, edges):
    g = _golden(name)
    lat = O.Lattice(str(g["lattice"]))
    shape = tuple(int(s) for s in g["shape"])
    bm, mm = _oracle_apply(lat, shape, _meshes(g, edges), g["prior_bc_mask"].copy(), g["prior_missing"].copy(), edges)
    sfx = "_edges" if edges else ""
    assert np.array_equal(bm, g["bc_mask" + sfx])
    assert np.array_equal(mm, g["missing_mask" + sfx])


def test_golden_cases_exercise_the_masker():
    """The fixtures hold solid voxels, marked cells and untouched prior marks."""
    for name in GOLDEN:
        g = _golden(name)
        bm, prior = g["bc_mask"][0], g["prior_bc_mask"][0]
        assert (bm == 255).sum() > 50
        ids = {int(g[f"mesh{k}_id"]) for k in range(int(g["n_mesh"]))}
        assert np.isin(bm, list(ids)).sum() > 50
        assert ((bm == prior) & (prior == 200)).sum() > 0
        # applied literally, the edge tests reject most of the surface voxels
        assert (g["bc_mask_edges"][0] == 255).sum() < (bm == 255).sum() / 3


def _soup(seed, shape, n_small=160):
    """Random triangles inside the domain: small ones, a few large, a few on
    integer coordinates and one degenerate."""
    rng = np.random.default_rng(seed)
    hi = np.array(shape, dtype=np.float64) - 1e-3
    centers = rng.uniform(1.0, hi - 1.0, size=(n_small, 1, 3))
    small = np.clip(centers + rng.uniform(-1.8, 1.8, size=(n_small, 3, 3)), 0.0, hi)
    big = rng.uniform(0.0, hi, size=(4, 3, 3))
    ints = rng.integers(0, np.array(shape) - 1, size=(6, 3, 3)).astype(np.float64)
    ints[:, :, 2] = ints[:, :1, 2]  # axis-aligned planes through voxel faces
    degenerate = np.array([[[1.0, 1.0, 1.0], [2.0, 2.0, 2.0], [3.0, 3.0, 3.0]]])
    return np.concatenate([small, big, ints, degenerate]).astype(np.float32)


def test_brick_pairs_cover_every_candidate():
    import torch

    from xlb_gb300.operator.boundary_masker.mesh_boundary_masker import brick_pairs

    shape = (21, 17, 13)
    tri = _soup(3, shape, 60)
    pdim = np.array(shape) + 2
    lo, hi = tri.min(axis=1), tri.max(axis=1)
    for brick in (1, 4, 8, 64):
        pt, pb = (x.numpy() for x in brick_pairs(torch.from_numpy(tri), shape, brick))
        nbd = (pdim + brick - 1) // brick
        assert pt.shape == pb.shape and pt.min() >= 0 and pt.max() < len(tri)
        assert pb.min() >= 0 and pb.max() < np.prod(nbd)
        have = set(zip(pt.tolist(), pb.tolist()))
        assert len(have) == len(pt)  # no repeats
        for b in range(int(np.prod(nbd))):
            bx, by, bz = b // (nbd[1] * nbd[2]), (b // nbd[2]) % nbd[1], b % nbd[2]
            p0 = np.array([bx, by, bz]) * brick
            p1 = np.minimum(p0 + brick, pdim) - 1  # voxels p0..p1 of the brick
            # a triangle's bounds meet some voxel [p - 1, p] of the brick iff lo <= p1 and hi >= p0 - 1
            need = np.nonzero(np.all((lo <= p1) & (hi >= p0 - 1), axis=1))[0]
            assert {(int(t), b) for t in need} <= have, (brick, b)


def test_brick_pairs_equal_the_direct_expansion():
    """Exactly the (triangle, brick) pairs whose bricks hold a voxel the
    triangle's bounds meet, each once (random soups, several brick sizes)."""
    import itertools

    import torch

    from xlb_gb300.operator.boundary_masker.mesh_boundary_masker import brick_pairs

    rng = np.random.default_rng(0)
    for trial in range(12):
        shape = tuple(int(v) for v in rng.integers(3, 30, 3))
        n = int(rng.integers(0, 60))
        hi = np.array(shape) - 1e-3
        tri = rng.uniform(0, 1, (n, 3, 3)) * hi
        if n:
            tri[: n // 2] = tri[: n // 2, :1] + rng.uniform(-0.5, 0.5, (n // 2, 3, 3))  # small ones
        tri = np.clip(tri, 0, hi).astype(np.float32)
        pdim = np.array(shape) + 2
        for brick in (1, 3, 8):
            pt, pb = brick_pairs(torch.from_numpy(tri), shape, brick)
            nbd = (pdim + brick - 1) // brick
            want = []
            for t in range(n):
                lo = np.maximum(np.ceil(tri[t].min(0).astype(np.float64)), 0).astype(int)
                up = np.minimum(np.floor(tri[t].max(0).astype(np.float64)) + 1, pdim - 1).astype(int)
                for bx, by, bz in itertools.product(*[range(lo[k] // brick, up[k] // brick + 1) for k in range(3)]):
                    want.append((t, int((bx * nbd[1] + by) * nbd[2] + bz)))
            assert sorted(zip(pt.tolist(), pb.tolist())) == sorted(want), (trial, brick)


def test_operator_checks_follow_xlb():
    import torch

    import xlb_gb300 as xlb
    from xlb_gb300.operator import boundary_condition as B
    from xlb_gb300.operator.boundary_masker import MeshBoundaryMasker

    pp = xlb.PrecisionPolicy.FP32FP32
    xlb.init(xlb.velocity_set.D2Q9(pp), xlb.ComputeBackend.CUDA, pp)
    with pytest.raises(NotImplementedError):
        MeshBoundaryMasker(xlb.velocity_set.D2Q9(pp), pp)
    vs = xlb.velocity_set.D3Q19(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    masker = MeshBoundaryMasker(vs, pp)
    bm = torch.zeros((1, 8, 8, 8), dtype=torch.uint8)
    mm = torch.zeros((19, 8, 8, 8), dtype=torch.bool)
    tri = np.array([[1.0, 1.0, 1.0], [5.0, 1.0, 1.0], [1.0, 5.0, 1.0]])
    with pytest.raises(AssertionError):
        masker(B.FullwayBounceBackBC(indices=[[1], [1], [1]]), bm, mm)  # no mesh_vertices
    with pytest.raises(AssertionError):
        masker(B.FullwayBounceBackBC(indices=[[1], [1], [1]], mesh_vertices=tri), bm, mm)
    with pytest.raises(AssertionError):
        masker(B.FullwayBounceBackBC(mesh_vertices=tri[:, :2]), bm, mm)
    with pytest.raises(ValueError, match="exceed domain"):
        masker(B.FullwayBounceBackBC(mesh_vertices=tri + 3.0), bm, mm)
    with pytest.raises(ValueError, match="exceed domain"):
        masker(B.FullwayBounceBackBC(mesh_vertices=tri - 1.5), bm, mm)
    assert not bm.any() and not mm.any()


# ----------------------------------------------------------------------------- GPU


def _gpu_apply(lat_name, bc_mask, missing, meshes, edges=False, brick=8):
    import torch

    import xlb_gb300 as xlb
    from xlb_gb300.operator.boundary_masker import MeshBoundaryMasker

    pp = xlb.PrecisionPolicy.FP32FP32
    vs = getattr(xlb.velocity_set, lat_name)(pp)
    masker = MeshBoundaryMasker(vs, pp, brick=brick, edge_tests=edges)
    bm = torch.from_numpy(bc_mask.copy()).cuda()
    mm = torch.from_numpy(missing.copy()).cuda()
    for verts, bid in meshes:
        masker.apply(verts if torch.is_tensor(verts) else np.asarray(verts, dtype=np.float32).reshape(-1, 3, 3), bid,
                     bm, mm)
    torch.cuda.synchronize()
    return bm.cpu().numpy(), mm.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("edges", [False, True])
@pytest.mark.parametrize("name", GOLDEN)
def test_gpu_matches_xlb_masker(name, edges):
    g = _golden(name)
    bm, mm = _gpu_apply(str(g["lattice"]), g["prior_bc_mask"], g["prior_missing"], _meshes(g, edges), edges)
    sfx = "_edges" if edges else ""
    assert np.array_equal(bm, g["bc_mask" + sfx])
    assert np.array_equal(mm, g["missing_mask" + sfx])


@pytest.mark.gpu
@pytest.mark.parametrize("brick", [1, 3, 8, 64])
@pytest.mark.parametrize("lattice", ["D3Q19", "D3Q27"])
def test_gpu_random_soup_matches_oracle(lattice, brick):
    shape = (29, 23, 19)
    lat = O.Lattice(lattice)
    tri = _soup(11, shape)
    rng = np.random.default_rng(5)
    prior_bm = np.where(rng.random((1,) + shape) < 0.04, 9, 0).astype(np.uint8)
    prior_mm = rng.random((lat.q,) + shape) < 0.02
    for edges in (False, True):
        want = _oracle_apply(lat, shape, [(tri, 17)], prior_bm.copy(), prior_mm.copy(), edges)
        got = _gpu_apply(lattice, prior_bm, prior_mm, [(tri, 17)], edges, brick)
        assert np.array_equal(got[0], want[0]), (edges, int((got[0] != want[0]).sum()))
        assert np.array_equal(got[1], want[1]), (edges, int((got[1] != want[1]).sum()))


@pytest.mark.gpu
def test_gpu_empty_mesh_leaves_masks():
    shape = (9, 8, 7)
    rng = np.random.default_rng(2)
    bm = rng.integers(0, 3, size=(1,) + shape).astype(np.uint8)
    mm = rng.random((19,) + shape) < 0.1
    got = _gpu_apply("D3Q19", bm, mm, [(np.zeros((0, 3, 3), np.float32), 4)])
    assert np.array_equal(got[0], bm) and np.array_equal(got[1], mm)


@pytest.mark.gpu
@pytest.mark.parametrize("lattice", ["D3Q19", "D3Q27"])
def test_stepper_with_mesh_bc_matches_oracle(lattice):
    """prepare_fields runs the indices masker, then the mesh masker; the masks
    and three FP32 steps on them equal the oracle's."""
    import torch

    import xlb_gb300 as xlb
    from xlb_gb300.operator import boundary_condition as B
    from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

    from _scenarios import faces, union

    shape = (20, 14, 12)
    pp = xlb.PrecisionPolicy.FP32FP32
    vs = getattr(xlb.velocity_set, lattice)(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    box = faces(shape, False)
    nob = faces(shape, True)
    walls = union(*[box[f] for f in ["bottom", "top", "front", "back"]])
    g = _golden("d3q19")
    body = g["mesh1_vertices"] + np.array([2.5, 1.0, 1.5])  # the icosahedron, moved into this grid
    bcs = [
        B.HalfwayBounceBackBC(indices=walls),
        B.EquilibriumBC(rho=1.0, u=(0.04, 0.0, 0.0), indices=nob["left"]),
        B.ExtrapolationOutflowBC(indices=nob["right"]),
        B.HalfwayBounceBackBC(mesh_vertices=body),
    ]
    stepper = IncompressibleNavierStokesStepper(xlb.grid.grid_factory(shape), bcs, collision_type="BGK")
    f_0, f_1, bc_mask, missing = stepper.prepare_fields()
    assert bcs[3].mesh_vertices is None  # the masker drops the vertices, as XLB's does

    lat = O.Lattice(lattice)
    obcs = [
        O.BC("halfway_bb", bcs[0].id, walls),
        O.BC("equilibrium", bcs[1].id, nob["left"], rho=1.0, u=(0.04, 0.0, 0.0)),
        O.BC("extrapolation", bcs[2].id, nob["right"]),
    ]
    obm, omm = O.masker(lat, shape, obcs)
    M.mask(lat, shape, body.astype(np.float32).reshape(-1, 3, 3), bcs[3].id, obm, omm)
    assert np.array_equal(bc_mask.cpu().numpy(), obm)
    assert np.array_equal(missing.cpu().numpy(), omm)
    assert (obm == bcs[3].id).sum() > 20 and (obm == 255).sum() > 10

    obcs.append(O.BC("halfway_bb", bcs[3].id, np.zeros((3, 0), dtype=np.int64)))
    store = O.Store("f32", lat)
    rng = np.random.default_rng(4)
    w = lat.w.reshape(-1, 1, 1, 1)
    f = (w * (1.0 + 0.05 * rng.uniform(-1, 1, size=(lat.q,) + shape))).astype(np.float32)
    want = O.run(lat, store, f.copy(), f.copy(), obm, omm, 1.6, obcs, 3, "BGK", np.float32)
    g0, g1 = torch.from_numpy(f).cuda(), torch.from_numpy(f.copy()).cuda()
    for i in range(3):
        g0, g1 = stepper(g0, g1, bc_mask, missing, 1.6, i)
        g0, g1 = g1, g0
    torch.cuda.synchronize()
    assert np.array_equal(g0.cpu().numpy(), want[0])
    assert np.array_equal(g1.cpu().numpy(), want[1])


@pytest.mark.gpu
def test_gpu_apply_accepts_torch_triangles():
    """Triangles as a host tensor or a CUDA tensor give the numpy path's marks."""
    import torch

    shape = (21, 17, 15)
    tri = _soup(21, shape, 60)
    prior_bm = np.zeros((1,) + shape, np.uint8)
    prior_mm = np.zeros((19,) + shape, bool)
    want = _gpu_apply("D3Q19", prior_bm, prior_mm, [(tri, 6)])
    for t in (torch.from_numpy(tri), torch.from_numpy(tri).cuda()):
        got = _gpu_apply("D3Q19", prior_bm, prior_mm, [(t, 6)])
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
