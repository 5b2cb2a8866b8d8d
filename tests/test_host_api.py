"""Host-side API (no GPU): velocity sets, precision policies, grid faces, BC
constructors, overlap checks, registry and the C-ABI descriptor."""

import itertools

import numpy as np
import pytest

import xlb_gb300 as xlb
from xlb_gb300 import _lib
from xlb_gb300.grid import grid_factory
from xlb_gb300.helper import check_bc_overlaps
from xlb_gb300.operator import boundary_condition as B
from xlb_gb300.operator.stepper.desc import make_desc
from xlb_gb300.precision_policy import Precision, PrecisionPolicy


@pytest.fixture
def d3q19_fp32():
    pp = PrecisionPolicy.FP32FP32
    vs = xlb.velocity_set.D3Q19(pp)
    xlb.init(vs, xlb.ComputeBackend.CUDA, pp)
    return vs


def test_velocity_set_tables():
    d2 = xlb.velocity_set.D2Q9()
    assert d2.c[0].tolist() == [0, 0, 0, 1, -1, 1, -1, 1, -1]
    assert d2.c[1].tolist() == [0, 1, -1, 0, 1, -1, 0, 1, -1]
    d27 = xlb.velocity_set.D3Q27()
    assert [tuple(v) for v in d27.c.T] == list(itertools.product([0, -1, 1], repeat=3))
    d19 = xlb.velocity_set.D3Q19()
    assert [tuple(v) for v in d19.c.T] == [v for v in itertools.product([0, -1, 1], repeat=3) if sum(map(abs, v)) <= 2]
    for vs in (d2, d19, d27):
        assert np.isclose(vs.w.sum(), 1.0)
        assert np.array_equal(vs.opp_indices[vs.opp_indices], np.arange(vs.q))
        assert np.array_equal(vs.c[:, vs.opp_indices], -vs.c)
        # second-order isotropy: sum_l w c_a c_b = delta_ab / 3
        m2 = np.einsum("l,al,bl->ab", vs.w, vs.c, vs.c)
        assert np.allclose(m2, np.eye(vs.d) / 3)


def test_d3q19_opposites_and_fast_axis_directions():
    vs = xlb.velocity_set.D3Q19()
    assert vs.opp_indices.tolist() == [0, 2, 1, 6, 8, 7, 3, 5, 4, 14, 16, 15, 18, 17, 9, 11, 10, 13, 12]
    assert np.nonzero(vs.c[2] == 1)[0].tolist() == [2, 5, 8, 11, 16]


def test_qi_and_cc():
    vs = xlb.velocity_set.D2Q9()
    assert vs.cc.shape == (9, 3) and vs.qi.shape == (9, 3)
    assert np.allclose(vs.qi[:, 0], vs.c[0] ** 2 - 1 / 3)
    assert np.allclose(vs.qi[:, 1], 2 * vs.c[0] * vs.c[1])


def test_precision_policies():
    assert PrecisionPolicy.FP32FP32.compute_precision == Precision.FP32
    assert PrecisionPolicy.FP64FP16.store_precision == Precision.FP16
    assert PrecisionPolicy.FP32BF16S.store_precision == Precision.BF16
    assert PrecisionPolicy.FP32FP16S.shifted and not PrecisionPolicy.FP32FP16.shifted
    assert PrecisionPolicy.FP32FP16S.store_bytes == 2 and PrecisionPolicy.FP64FP64.store_bytes == 8


def test_bounding_box_indices_3d():
    g = grid_factory((5, 6, 7), device="cpu")
    box = g.bounding_box_indices()
    nob = g.bounding_box_indices(remove_edges=True)
    top = np.array(box["top"])
    assert np.all(top[2] == 6) and top.shape == (3, 5 * 6)
    left = np.array(nob["left"])
    assert np.all(left[0] == 0) and left.shape == (3, 4 * 5)
    assert set(box) == {"bottom", "top", "left", "right", "front", "back"}


def test_bounding_box_indices_2d():
    g = grid_factory((5, 6), device="cpu")
    box = g.bounding_box_indices()
    assert np.all(np.array(box["top"])[1] == 5)
    assert np.array(g.bounding_box_indices(remove_edges=True)["right"]).shape == (2, 4)


def test_zouhe_prescribed_value_rules(d3q19_fp32):
    bc = B.ZouHeBC("velocity", prescribed_value=(0.0, -0.03, 0.0), indices=[[0], [1], [1]])
    assert bc.prescribed_value == -0.03
    with pytest.raises(ValueError):
        B.ZouHeBC("velocity", prescribed_value=(0.01, 0.02, 0.0), indices=[[0], [1], [1]])
    with pytest.raises(ValueError):
        B.ZouHeBC("velocity", prescribed_value=0.1, indices=[[0], [1], [1]])
    with pytest.raises(ValueError):
        B.ZouHeBC("vorticity", prescribed_value=1.0)
    p = B.RegularizedBC("pressure", prescribed_value=1.01, indices=[[0], [1], [1]])
    assert p.kind == _lib.BC_REGULARIZED_PRESSURE and p.needs_aux_recovery and p.needs_padding


def test_registry_ids_increase(d3q19_fp32):
    a = B.FullwayBounceBackBC(indices=[[0], [0], [0]])
    b = B.HalfwayBounceBackBC(indices=[[1], [1], [1]])
    assert (a.id, b.id) == (1, 2)


def test_overlap_checks(d3q19_fp32):
    a = B.FullwayBounceBackBC(indices=[[0, 1], [0, 0], [0, 0]])
    b = B.HalfwayBounceBackBC(indices=[[1], [0], [0]])
    with pytest.raises(ValueError):
        check_bc_overlaps([a, b], 3)
    c = B.FullwayBounceBackBC(indices=[[2, 2], [0, 0], [0, 0]])
    with pytest.raises(ValueError):
        check_bc_overlaps([c], 3)
    check_bc_overlaps([a], 3)


def test_mesh_vertices_kept_for_the_mesh_masker(d3q19_fp32):
    v = np.zeros((3, 3))
    bc = B.HalfwayBounceBackBC(mesh_vertices=v)
    assert bc.mesh_vertices is v and bc.indices is None
    check_bc_overlaps([bc], 3)  # BCs without indices take no part in the overlap check


def test_extrapolation_global_normal(d3q19_fp32):
    g = grid_factory((8, 6, 6), device="cpu")
    out = B.ExtrapolationOutflowBC(indices=g.bounding_box_indices(remove_edges=True)["right"])
    assert out.normal.tolist() == [1, 0, 0]
    inl = B.ExtrapolationOutflowBC(indices=g.bounding_box_indices(remove_edges=True)["left"])
    assert inl.normal.tolist() == [-1, 0, 0]


def test_desc(d3q19_fp32):
    eq = B.EquilibriumBC(rho=1.0, u=(0.05, 0.0, 0.0), indices=[[1], [1], [5]])
    fw = B.FullwayBounceBackBC(indices=[[0], [0], [0]])
    d = make_desc(d3q19_fp32, PrecisionPolicy.FP32FP32, (8, 8, 6), _lib.BGK, [eq, fw])
    assert (d.lattice, d.store, d.compute, d.nbc, d.nx, d.nz) == (1, 0, 0, 2, 8, 6)
    assert d.bc[0].kind == _lib.BC_EQUILIBRIUM and d.bc[0].u[0] == 0.05
    assert d.bc[1].kind == _lib.BC_FULLWAY_BB


def test_stepper_rejects_kbc_d3q19(d3q19_fp32):
    from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

    with pytest.raises(NotImplementedError):
        IncompressibleNavierStokesStepper(grid_factory((4, 4, 4), device="cpu"), [], collision_type="KBC")
    with pytest.raises(ValueError):
        IncompressibleNavierStokesStepper(grid_factory((4, 4, 4), device="cpu"), [], streaming_scheme="push")


@pytest.mark.gpu
def test_stepper_checks_each_argument_position(d3q19_fp32):
    """The stepper skips its field checks for tensors it has already accepted in
    the same argument position; a tensor accepted as f_0 is still rejected as
    bc_mask, and a reshaped or re-pointed tensor is checked again."""
    import torch

    from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

    grid = grid_factory((12, 10, 8))
    st = IncompressibleNavierStokesStepper(grid, [], collision_type="BGK")
    f_0, f_1, bc_mask, missing_mask = st.prepare_fields()
    for i in range(3):
        f_0, f_1 = st(f_0, f_1, bc_mask, missing_mask, 1.6, i)
        f_0, f_1 = f_1, f_0
    with pytest.raises((TypeError, ValueError)):
        st(f_0, f_1, f_0, missing_mask, 1.6, 3)
    with pytest.raises((TypeError, ValueError)):
        st(f_0, f_1, bc_mask, f_1, 1.6, 3)
    with pytest.raises(ValueError):
        st(f_0, f_1, bc_mask, missing_mask.view(missing_mask.shape[0], -1), 1.6, 3)
    small = torch.empty((f_1.shape[0], 2, 10, 8), dtype=f_1.dtype, device=f_1.device)
    f_1.set_(small)
    with pytest.raises(ValueError):
        st(f_0, f_1, bc_mask, missing_mask, 1.6, 3)
    torch.cuda.synchronize()
