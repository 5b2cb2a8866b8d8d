"""Fused CUDA step vs the CPU oracle on identical inputs.

The kernels are built with --fmad=false and keep the oracle's operation order,
so for every precision policy the comparison is exact (bit-for-bit up to the
sign of zero): FP32 against the float32 oracle, FP64 against the float64
oracle, and the FP16/BF16 store forms against the oracle's identical rounding.
"""

import numpy as np
import pytest

from _scenarios import Scenario

CASES = [
    # lattice, shape, layout, collision
    ("D2Q9", (24, 20), "cavity_fullway", "BGK"),
    ("D2Q9", (24, 20), "cavity_halfway", "BGK"),
    ("D2Q9", (30, 18), "channel_zouhe", "BGK"),
    ("D2Q9", (30, 18), "channel_regularized", "BGK"),
    ("D2Q9", (30, 18), "channel_pressure", "BGK"),
    ("D2Q9", (24, 20), "periodic", "KBC"),
    ("D2Q9", (30, 18), "channel_regularized", "KBC"),
    ("D3Q19", (12, 10, 9), "cavity_fullway", "BGK"),
    ("D3Q19", (12, 10, 9), "cavity_halfway", "BGK"),
    ("D3Q19", (16, 10, 10), "channel_zouhe", "BGK"),
    ("D3Q19", (16, 10, 10), "channel_regularized", "BGK"),
    ("D3Q19", (14, 9, 8), "channel_pressure", "BGK"),
    ("D3Q27", (12, 10, 9), "cavity_fullway", "BGK"),
    ("D3Q27", (16, 10, 10), "channel_regularized", "KBC"),
    ("D3Q27", (12, 10, 9), "periodic", "KBC"),
    ("D3Q27", (16, 10, 10), "channel_zouhe", "KBC"),
]


def _compare(got, want, what):
    assert got.shape == want.shape, what
    if not np.array_equal(got, want):
        g = got.astype(np.float64)
        w = want.astype(np.float64)
        bad = np.argwhere(g != w)
        raise AssertionError(
            f"{what}: {len(bad)} of {g.size} values differ; first at {tuple(bad[0])}: "
            f"{g[tuple(bad[0])]!r} vs {w[tuple(bad[0])]!r}; max |diff| {np.max(np.abs(g - w)):.3e}"
        )


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64"])
@pytest.mark.parametrize("lattice,shape,layout,collision", CASES)
def test_step_matches_oracle(lattice, shape, layout, collision, policy):
    sc = Scenario(lattice, shape, layout, policy=policy, collision=collision)
    sc.randomize(seed=1)
    steps = 4
    want0, want1 = sc.oracle_steps(steps)
    got0, got1 = sc.gpu_steps(steps)
    _compare(got0, want0, "f_0 (newest state)")
    _compare(got1, want1, "f_1 (previous buffer incl. aux recovery)")


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["f16", "f16s", "bf16s", "fp64f32", "fp64f16"])
@pytest.mark.parametrize(
    "lattice,shape,layout,collision",
    [
        ("D2Q9", (30, 18), "channel_regularized", "BGK"),
        ("D3Q19", (16, 10, 10), "channel_zouhe", "BGK"),
        ("D3Q19", (12, 10, 9), "cavity_fullway", "BGK"),
        ("D3Q27", (16, 10, 10), "channel_regularized", "KBC"),
    ],
)
def test_store_forms_match_oracle(lattice, shape, layout, collision, policy):
    sc = Scenario(lattice, shape, layout, policy=policy, collision=collision)
    sc.randomize(seed=2)
    want0, want1 = sc.oracle_steps(3)
    got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


@pytest.mark.gpu
def test_run_equals_step_loop():
    """xlbg_run (swap inside C) == the Python swap loop, odd and even step counts."""
    sc = Scenario("D3Q19", (16, 10, 10), "channel_regularized", policy="fp32")
    sc.randomize(seed=3)
    for steps in (3, 4):
        a = sc.gpu_steps(steps)
        b = sc.gpu_steps(steps, use_run=True)
        _compare(b[0], a[0], f"run f_0 ({steps})")
        _compare(b[1], a[1], f"run f_1 ({steps})")


@pytest.mark.gpu
def test_skip_cells_untouched():
    """Cells with id 255 are skipped: their f_1 keeps its content (nse_stepper.py:356-358)."""
    sc = Scenario("D3Q19", (12, 10, 9), "cavity_fullway", policy="fp32")
    sc.randomize(seed=4)
    sc.bc_mask[0, 5:7, 4:6, 3:5] = 255
    want0, want1 = sc.oracle_steps(3)
    got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


@pytest.mark.gpu
@pytest.mark.parametrize(
    "lattice,shape,layout",
    [("D2Q9", (30, 18), "channel_zouhe"), ("D3Q19", (16, 10, 10), "channel_regularized"), ("D3Q27", (12, 10, 9), "cavity_halfway")],
)
def test_prepare_fields_matches_oracle(lattice, shape, layout):
    """Masker (bc_mask, missing_mask), equilibrium initialisation and aux data."""
    sc = Scenario(lattice, shape, layout, policy="fp32")
    f_0, f_1, bc_mask, missing = sc.stepper.prepare_fields()
    _compare(bc_mask.cpu().numpy(), sc.bc_mask, "bc_mask")
    _compare(missing.cpu().numpy(), sc.missing, "missing_mask")
    _compare(sc.to_numpy(f_0), sc.f0, "f_0 init")
    _compare(sc.to_numpy(f_1), sc.f1, "f_1 init with aux")


# Shapes whose contiguous extent (nz, or ny in 2D) is divisible by 2 and 4, so the
# V-cells-per-thread kernel runs (V = 2 for 4/8-byte stores, V = 4 for 2-byte
# stores), with several warps per row and a partial last warp.
VEC_CASES = [
    ("D3Q19", (6, 5, 136), "cavity_fullway"),
    ("D3Q19", (8, 6, 68), "channel_regularized"),
    ("D3Q19", (7, 6, 264), "channel_zouhe"),
    ("D2Q9", (10, 260), "channel_zouhe"),
    ("D2Q9", (9, 1028), "cavity_halfway"),
    ("D3Q27", (6, 5, 40), "cavity_halfway"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64", "f16s", "bf16s", "f16"])
@pytest.mark.parametrize("lattice,shape,layout", VEC_CASES)
def test_vector_kernel_matches_oracle(lattice, shape, layout, policy):
    sc = Scenario(lattice, shape, layout, policy=policy, collision="BGK")
    sc.randomize(seed=7)
    want0, want1 = sc.oracle_steps(3)
    got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "f16s"])
def test_vector_kernel_skip_cells(policy):
    sc = Scenario("D3Q19", (6, 5, 136), "cavity_fullway", policy=policy)
    sc.randomize(seed=8)
    sc.bc_mask[0, 2:4, 1:3, 37:71] = 255
    want0, want1 = sc.oracle_steps(2)
    got0, got1 = sc.gpu_steps(2)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["fp32", "fp64", "f16", "f16s", "bf16s"])
@pytest.mark.parametrize(
    "lattice,shape,layout",
    [("D2Q9", (30, 18), "channel_zouhe"), ("D3Q19", (16, 10, 10), "channel_regularized"),
     ("D3Q19", (6, 5, 136), "cavity_fullway"), ("D3Q27", (12, 10, 9), "cavity_halfway")],
)
def test_bgk_pair_form_matches_oracle(lattice, shape, layout, policy):
    """collision_type="BGK_PAIR" (pair form on f) under every policy; the shifted
    policies default to BGK on the stored deviations instead."""
    sc = Scenario(lattice, shape, layout, policy=policy, collision="BGK_PAIR")
    sc.randomize(seed=9)
    want0, want1 = sc.oracle_steps(3)
    got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


TMA_CASES = [
    # contiguous axis a multiple of 8: the 16-bit stores take the TMA-staged kernel
    ("D3Q19", (10, 8, 16), "channel_zouhe"),
    ("D3Q19", (10, 8, 16), "channel_regularized"),
    ("D3Q19", (6, 5, 264), "cavity_fullway"),  # two tensor copies per row, the second partly outside
    ("D3Q19", (4, 3, 520), "periodic"),  # shifted stores: three segments; raw FP16: marching kernel
    ("D2Q9", (30, 24), "channel_regularized"),
    ("D3Q27", (10, 8, 16), "channel_pressure"),
    ("D3Q27", (6, 5, 256), "cavity_halfway"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["f16", "f16s", "bf16s"])
@pytest.mark.parametrize("lattice,shape,layout", TMA_CASES)
def test_tma_staged_step_matches_oracle(lattice, shape, layout, policy):
    from xlb_gb300 import _lib

    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=12)
    if layout == "periodic":
        sc.bc_mask[0, 1:3, 0:2, 100:140] = 255  # skip cells inside staged rows
        sc.bc_mask[0, 0, 1:3, 201:206] = 255  # odd bounds: cell pairs with one skip cell
    want0, want1 = sc.oracle_steps(3)
    got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")
    assert _lib.load().xlbg_device_faults(1) == 0


SEG_CASES = [
    # segments of 256 cells of the contiguous axis
    ("D3Q19", (10, 8, 16), "channel_zouhe"),  # one segment: both aprons wrap
    ("D3Q19", (10, 8, 16), "channel_regularized"),
    ("D3Q19", (6, 5, 264), "cavity_fullway"),  # segments of 256 and 8
    ("D3Q19", (4, 3, 520), "periodic"),  # 256, 256, 8; skip cells across segment ends
    ("D3Q19", (3, 4, 1032), "periodic"),  # longer than any full-row stage
    ("D2Q9", (30, 24), "channel_regularized"),
    ("D2Q9", (12, 528), "cavity_fullway"),
    ("D3Q27", (10, 8, 16), "channel_pressure"),
    ("D3Q27", (4, 3, 768), "cavity_halfway"),
    ("D3Q19", (6, 5, 8), "periodic"),  # the shortest row: one 8-cell segment, both aprons wrapped
    ("D3Q27", (5, 4, 24), "channel_regularized"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["auto", "tma_wide"])
@pytest.mark.parametrize("policy", ["f16s", "bf16s", "f16sr", "bf16sr"])
@pytest.mark.parametrize("lattice,shape,layout", SEG_CASES)
def test_segmented_step_matches_oracle(lattice, shape, layout, policy, kernel):
    """The segmented two-cell kernel of the shifted stores (rows staged as
    256-cell segments with 16-byte aprons), with 32- and 64-bit plane offsets,
    bit for bit against the oracle."""
    from xlb_gb300 import _lib

    sel = _lib.KERNEL_AUTO if kernel == "auto" else _lib.KERNEL_TMA_WIDE
    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=19)
    if layout == "periodic":
        sc.bc_mask[0, 1:3, 0:2, 250:262] = 255  # skip cells across the first segment end
        sc.bc_mask[0, 0, 1:3, 509:514] = 255  # odd bounds: cell pairs with one skip cell
    want0, want1 = sc.oracle_steps(3)
    with _lib.forced_kernel(sel):
        got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")
    assert _lib.load().xlbg_device_faults(1) == 0


VARIANT_CASES = [
    ("D2Q9", (30, 18), "channel_regularized"),
    ("D3Q19", (16, 10, 10), "channel_zouhe"),
    ("D3Q19", (12, 10, 9), "cavity_fullway"),
    ("D3Q27", (10, 8, 16), "channel_pressure"),
    ("D3Q19", (6, 5, 264), "cavity_fullway"),
    ("D3Q19", (10, 8, 16), "channel_regularized"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["march", "march_wide", "cell", "tma_wide"])
@pytest.mark.parametrize("policy", ["fp32", "f16s", "bf16s", "f16"])
@pytest.mark.parametrize("lattice,shape,layout", VARIANT_CASES)
def test_kernel_variants_match_oracle(lattice, shape, layout, policy, kernel):
    """Kernel variants the automatic choice takes only on grids too large for a
    test, or not on these shapes, forced through xlbg_debug_force_kernel: the
    marching kernel with 32- and 64-bit plane offsets (64-bit when Q x cells >=
    2^32, e.g. 1024 x 1024 x 768 D3Q19), the one-cell-per-thread kernel (grids
    of 2^31 cells and more), and the TMA-staged kernel with 64-bit plane
    offsets (the 16-bit stores on grids with Q x cells >= 2^32)."""
    from xlb_gb300 import _lib

    sel = {"march": _lib.KERNEL_MARCH, "march_wide": _lib.KERNEL_MARCH_WIDE, "cell": _lib.KERNEL_CELL,
           "tma_wide": _lib.KERNEL_TMA_WIDE}[kernel]
    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=14)
    want0, want1 = sc.oracle_steps(3)
    with _lib.forced_kernel(sel):
        got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")
    assert _lib.load().xlbg_device_faults(1) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,layout", [
    ("D2Q9", (30, 18), "channel_regularized"),
    ("D2Q9", (24, 20), "cavity_fullway"),
    ("D3Q19", (16, 10, 10), "channel_zouhe"),
    ("D3Q19", (12, 10, 9), "cavity_halfway"),
    ("D3Q19", (14, 9, 8), "channel_pressure"),
    ("D3Q27", (16, 10, 10), "channel_regularized"),
    ("D3Q19", (6, 5, 136), "cavity_fullway"),
])
def test_fp32_deviation_form_matches_oracle(lattice, shape, layout):
    """collision_type="BGK_SHIFTED" with FP32 storage: BGK on g = f - w_l, bit
    for bit against the oracle's restatement."""
    sc = Scenario(lattice, shape, layout, policy="fp32", collision="BGK_SHIFTED")
    sc.randomize(seed=15)
    want0, want1 = sc.oracle_steps(4)
    got0, got1 = sc.gpu_steps(4)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")


KBC_TMA_CASES = [
    # FP32 D3Q27 KBC with a contiguous axis of 8..512 cells (4-byte multiples of 16 bytes):
    # the TMA-staged kernel, staged rows of 192, 256 and 512 cells
    ("D3Q27", (10, 8, 16), "channel_regularized"),
    ("D3Q27", (10, 8, 16), "channel_zouhe"),
    ("D3Q27", (6, 5, 192), "periodic"),
    ("D3Q27", (5, 4, 264), "cavity_halfway"),
    ("D3Q27", (6, 5, 200), "channel_pressure"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["auto", "tma_wide"])
@pytest.mark.parametrize("lattice,shape,layout", KBC_TMA_CASES)
def test_kbc_fp32_tma_matches_oracle(lattice, shape, layout, kernel):
    from xlb_gb300 import _lib

    sc = Scenario(lattice, shape, layout, policy="fp32", collision="KBC")
    sc.randomize(seed=16)
    if layout == "periodic":
        sc.bc_mask[0, 1:3, 0:2, 100:140] = 255  # skip cells inside staged rows
    want0, want1 = sc.oracle_steps(3)
    with _lib.forced_kernel(_lib.KERNEL_AUTO if kernel == "auto" else _lib.KERNEL_TMA_WIDE):
        got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")
    assert _lib.load().xlbg_device_faults(1) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["auto", "march", "cell", "tma_wide"])
@pytest.mark.parametrize("policy", ["f16sr", "bf16sr"])
@pytest.mark.parametrize("lattice,shape,layout", [
    ("D3Q19", (10, 8, 16), "channel_regularized"),
    ("D3Q19", (6, 5, 264), "cavity_fullway"),
    ("D2Q9", (30, 16), "channel_zouhe"),
    ("D3Q27", (10, 8, 16), "channel_pressure"),
    ("D3Q19", (12, 10, 9), "cavity_halfway"),
])
def test_stochastic_rounding_matches_oracle(lattice, shape, layout, policy, kernel):
    """FP32FP16SR / FP32BF16SR: BGK on the stored deviations with every store
    rounded stochastically (cvt.rs, random bits hashed from the cell index and
    the timestep argument), bit for bit against the oracle's restatement of
    cvt.rs and of the hash, on every kernel variant."""
    from xlb_gb300 import _lib

    sel = {"auto": _lib.KERNEL_AUTO, "march": _lib.KERNEL_MARCH, "cell": _lib.KERNEL_CELL,
           "tma_wide": _lib.KERNEL_TMA_WIDE}[kernel]
    sc = Scenario(lattice, shape, layout, policy=policy)
    sc.randomize(seed=17)
    want0, want1 = sc.oracle_steps(3)
    with _lib.forced_kernel(sel):
        got0, got1 = sc.gpu_steps(3)
    _compare(got0, want0, "f_0")
    _compare(got1, want1, "f_1")
    assert _lib.load().xlbg_device_faults(1) == 0


@pytest.mark.gpu
def test_stochastic_rounding_run_uses_the_timesteps():
    """xlbg_run seeds step k with timestep0 + k, like the per-step loop."""
    sc = Scenario("D3Q19", (10, 8, 16), "channel_regularized", policy="f16sr")
    sc.randomize(seed=18)
    a = sc.gpu_steps(4)
    b = sc.gpu_steps(4, use_run=True)
    _compare(b[0], a[0], "run f_0")
    _compare(b[1], a[1], "run f_1")


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,shape,layout,policy,collision", [
    ("D2Q9", (30, 18), "channel_zouhe", "fp32", "BGK"),
    ("D3Q19", (16, 10, 10), "channel_regularized", "fp32", "BGK"),
    ("D3Q19", (10, 8, 16), "cavity_fullway", "f16s", "BGK"),
    ("D3Q27", (10, 8, 16), "channel_regularized", "fp32", "KBC"),
    ("D3Q19", (12, 10, 9), "cavity_halfway", "fp64", "BGK"),
])
def test_run_longer_loops_equal_step_loop(lattice, shape, layout, policy, collision):
    """xlbg_run over 11 steps (an odd count: the result is in the other buffer)
    equals the oracle, and 11 more on the same buffers equal 22 per-step calls,
    bit for bit."""
    import torch

    sc = Scenario(lattice, shape, layout, policy=policy, collision=collision)
    sc.randomize(seed=21)
    want0, want1 = sc.oracle_steps(11)
    f_0, f_1, bcm, mm = sc.gpu_fields()
    f_0, f_1 = sc.stepper.run(f_0, f_1, bcm, mm, sc.omega, 11)
    torch.cuda.synchronize()
    _compare(sc.to_numpy(f_0), want0, "f_0 after 11")
    _compare(sc.to_numpy(f_1), want1, "f_1 after 11")
    f_0, f_1 = sc.stepper.run(f_0, f_1, bcm, mm, sc.omega, 11)
    g_0, g_1, gbcm, gmm = sc.gpu_fields()
    for i in range(22):
        g_0, g_1 = sc.stepper(g_0, g_1, gbcm, gmm, sc.omega, i)
        g_0, g_1 = g_1, g_0
    torch.cuda.synchronize()
    _compare(sc.to_numpy(f_0), sc.to_numpy(g_0), "f_0 after 22")
    _compare(sc.to_numpy(f_1), sc.to_numpy(g_1), "f_1 after 22")
