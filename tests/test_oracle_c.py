"""The C restatement (oracle/lbm_ref.c) and the numpy oracle agree bit for bit
(FP32 and FP64), so either can serve as the checker."""

import numpy as np
import pytest

from oracle import cref
from oracle import lbm_oracle as O
from _scenarios import Scenario


@pytest.mark.parametrize("policy", ["fp32", "fp64"])
@pytest.mark.parametrize(
    "lattice,shape,layout,collision",
    [
        ("D2Q9", (30, 18), "channel_zouhe", "BGK"),
        ("D2Q9", (30, 18), "channel_regularized", "KBC"),
        ("D3Q19", (12, 10, 9), "cavity_fullway", "BGK"),
        ("D3Q19", (16, 10, 10), "channel_regularized", "BGK"),
        ("D3Q19", (14, 9, 8), "channel_pressure", "BGK"),
        ("D3Q27", (16, 10, 10), "channel_zouhe", "KBC"),
        ("D3Q27", (12, 10, 9), "cavity_halfway", "BGK"),
    ],
)
def test_c_oracle_equals_numpy_oracle(lattice, shape, layout, collision, policy):
    sc = Scenario(lattice, shape, layout, policy=policy, collision=collision)
    sc.randomize(seed=5)
    want0, want1 = sc.oracle_steps(4)
    st = cref.Stepper(sc.lat, shape, sc.bc_mask, sc.missing, sc.obcs, collision, sc.T, threads=2)
    got0, got1 = st.run(sc.f0.copy(), sc.f1.copy(), sc.omega, 4)
    assert np.array_equal(got0, want0)
    assert np.array_equal(got1, want1)


def test_c_oracle_skip_cells():
    sc = Scenario("D3Q19", (12, 10, 9), "cavity_fullway", policy="fp32")
    sc.randomize(seed=6)
    sc.bc_mask[0, 5:7, 4:6, 3:5] = 255
    want0, want1 = sc.oracle_steps(2)
    st = cref.Stepper(sc.lat, sc.shape, sc.bc_mask, sc.missing, sc.obcs, "BGK", sc.T)
    got0, got1 = st.run(sc.f0.copy(), sc.f1.copy(), sc.omega, 2)
    assert np.array_equal(got0, want0) and np.array_equal(got1, want1)
    assert O is not None


@pytest.mark.parametrize("lattice,shape,layout", [("D3Q19", (16, 10, 10), "channel_regularized"), ("D2Q9", (30, 18), "channel_zouhe")])
def test_c_oracle_pair_form(lattice, shape, layout):
    sc = Scenario(lattice, shape, layout, policy="fp32", collision="BGK_PAIR")
    sc.randomize(seed=12)
    want0, want1 = sc.oracle_steps(3)
    st = cref.Stepper(sc.lat, shape, sc.bc_mask, sc.missing, sc.obcs, "BGK_PAIR", sc.T, threads=2)
    got0, got1 = st.run(sc.f0.copy(), sc.f1.copy(), sc.omega, 3)
    assert np.array_equal(got0, want0) and np.array_equal(got1, want1)


@pytest.mark.parametrize("policy", ["fp32", "fp64"])
@pytest.mark.parametrize(
    "lattice,shape,layout",
    [("D3Q19", (6, 5, 70), "cavity_fullway"), ("D3Q19", (8, 6, 72), "channel_regularized"),
     ("D3Q27", (5, 4, 68), "periodic"), ("D2Q9", (12, 100), "channel_zouhe")],
)
def test_c_oracle_fluid_chunks(lattice, shape, layout, policy):
    """Rows long enough for the C restatement's vectorised fluid chunks (32 fluid
    cells away from the row ends) still equal the numpy oracle bit for bit."""
    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=8)
    if layout == "periodic":
        sc.bc_mask[0, 1:3, 1:3, 20:23] = 255  # skip cells inside a chunk: that chunk runs per cell
    want0, want1 = sc.oracle_steps(3)
    st = cref.Stepper(sc.lat, sc.shape, sc.bc_mask, sc.missing, sc.obcs, "BGK", sc.T, threads=2)
    got0, got1 = st.run(sc.f0.copy(), sc.f1.copy(), sc.omega, 3)
    assert np.array_equal(got0, want0)
    assert np.array_equal(got1, want1)
