"""The oracle against XLB's own unit-test expectations and equation-level known answers.

XLB ships no golden files; its tests (tests/ in the XLB tree) pin analytic results:
stream == roll, BGK formula, feq at rest, moments of feq, bounce-back and
equilibrium BC values, masker ids.  Each test below restates one of those on the
oracle, plus conservation and BC identities that follow from the equations.
"""

import numpy as np
import pytest

from oracle import lbm_oracle as O

LATS = ["D2Q9", "D3Q19", "D3Q27"]


def shape_for(lat, n=10):
    return (n, n + 2) if lat == "D2Q9" else (n, n + 1, n - 1)


def s3(shape):
    return tuple(shape) if len(shape) == 3 else tuple(shape) + (1,)


@pytest.mark.parametrize("lat", LATS)
def test_stream_is_roll(lat):
    """tests/kernels/stream/test_stream_warp.py:32-77: pull stream == roll by c_l."""
    L = O.Lattice(lat)
    shp = s3(shape_for(lat))
    f = np.zeros((L.q,) + shp)
    f[..., shp[-1] // 2] = 1.0
    f[:, 1, 2, ...] = 3.0  # something near an edge
    got = O.pull(L, f)
    # explicit per-cell pull with XLB's one-cell wrap (stream.py:64-82)
    want = np.empty_like(f)
    for l in range(L.q):
        for idx in np.ndindex(*shp):
            src = list(idx)
            for d in range(L.d):
                v = idx[d] - L.c[d, l]
                src[d] = shp[d] - 1 if v < 0 else (0 if v >= shp[d] else v)
            want[(l,) + idx] = f[(l,) + tuple(src)]
    assert np.array_equal(got, want)


@pytest.mark.parametrize("lat", LATS)
@pytest.mark.parametrize("omega", [0.6, 1.0])
def test_bgk_formula(lat, omega):
    """tests/kernels/collision/test_bgk_collision_warp.py:112-134."""
    L = O.Lattice(lat)
    rng = np.random.default_rng(0)
    f = rng.random((L.q, 50))
    feq = rng.random((L.q, 50))
    assert np.allclose(O.bgk(f, feq, omega), f - omega * (f - feq), atol=1e-5)


@pytest.mark.parametrize("lat", LATS)
def test_equilibrium_at_rest(lat):
    """tests/kernels/equilibrium/test_equilibrium_warp.py:168-187: sum feq = 1, feq_i = w_i."""
    L = O.Lattice(lat)
    n = 7
    feq = O.equilibrium(L, np.ones(n), [np.zeros(n)] * L.d, np.float64)
    assert np.allclose(feq.sum(axis=0), 1.0)
    for i in range(L.q):
        assert np.allclose(feq[i], L.w[i])


@pytest.mark.parametrize("lat", LATS)
@pytest.mark.parametrize("rho,vel", [(1.0, 0.0), (1.1, 1.0), (1.1, 2.0)])
def test_macroscopic_of_equilibrium(lat, rho, vel):
    """tests/kernels/macroscopic/test_macroscopic_warp.py:216-245."""
    L = O.Lattice(lat)
    n = 5
    feq = O.equilibrium(L, np.full(n, rho), [np.full(n, vel)] * L.d, np.float64)
    r, u = O.macroscopic(L, feq, np.float64)
    assert np.allclose(r, rho)
    for d in range(L.d):
        assert np.allclose(u[d], vel, atol=1e-6)


def _ball(shape, radius):
    grids = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    r2 = sum((g - s // 2) ** 2 for g, s in zip(grids, shape))
    return np.array(np.where(r2 < radius**2))


@pytest.mark.parametrize("lat", LATS)
def test_masker_ids(lat):
    """tests/boundary_conditions/mask/test_bc_indices_masker_warp.py:220-277."""
    L = O.Lattice(lat)
    shape = (20,) * (2 if lat == "D2Q9" else 3)
    idx = _ball(shape, 5)
    bcm, miss = O.masker(L, shape, [O.BC("fullway_bb", 5, idx)])
    assert bcm.shape == (1,) + s3(shape) and bcm.dtype == np.uint8
    assert miss.shape == (L.q,) + s3(shape) and miss.dtype == bool
    sel = tuple(idx) if lat != "D2Q9" else (idx[0], idx[1], 0)
    assert np.all(bcm[0][sel] == 5)
    bcm[0][sel] = 0
    assert np.all(bcm == 0)
    assert not miss.any()  # interior, no padding for fullway: nothing missing


@pytest.mark.parametrize("lat", LATS)
def test_masker_padding_marks_push_neighbours(lat):
    """indices_boundary_masker.py:152-156: interior padding BCs mark x + c_l as missing in l."""
    L = O.Lattice(lat)
    shape = (16,) * (2 if lat == "D2Q9" else 3)
    idx = _ball(shape, 3)
    bcm, miss = O.masker(L, shape, [O.BC("halfway_bb", 7, idx)])
    solid = np.zeros(s3(shape), dtype=bool)
    solid[tuple(idx) if lat != "D2Q9" else (idx[0], idx[1], 0)] = True
    for l in range(L.q):
        shifted = O.pull(L, solid[None].repeat(L.q, 0))[l]  # solid(x - c_l)
        assert np.array_equal(miss[l], shifted), l
    assert np.array_equal(bcm[0] == 7, miss.any(axis=0))


@pytest.mark.parametrize("lat", LATS)
def test_fullway_and_equilibrium_bc_in_step(lat):
    """tests/boundary_conditions/*: inside the BC set, fullway gives f_pre[opp]; the
    equilibrium BC gives w at rho=1, u=0; outside the sets nothing else changes."""
    L = O.Lattice(lat)
    shape = shape_for(lat, 12)
    st = O.Store("f64", L)
    rng = np.random.default_rng(1)
    f0 = (L.w.reshape((-1,) + (1,) * 3) * (1 + 0.1 * rng.uniform(-1, 1, (L.q,) + s3(shape))))
    ball = _ball(shape, 3)
    eq_idx = np.array([[1, 2], [1, 1]] + ([[1, 1]] if len(shape) == 3 else []))
    bcs = [O.BC("fullway_bb", 1, ball), O.BC("equilibrium", 2, eq_idx, rho=1.0, u=(0, 0, 0))]
    bcm, miss = O.masker(L, shape, bcs)
    _, f1 = O.step(L, st, f0, f0.copy(), bcm, miss, 1.3, bcs)
    fps = O.pull(L, f0)
    m = bcm[0] == 1
    assert np.array_equal(f1[:, m], fps[:, m][L.opp])
    e = bcm[0] == 2
    assert np.allclose(f1[:, e], L.w[:, None], atol=1e-15)


@pytest.mark.parametrize("lat", LATS)
@pytest.mark.parametrize("coll", ["BGK", "KBC"])
def test_collision_invariants(lat, coll):
    """BGK and KBC conserve mass and momentum per cell."""
    if coll == "KBC" and lat == "D3Q19":
        pytest.skip("KBC is defined for D2Q9 and D3Q27 only (kbc.py:184-185)")
    L = O.Lattice(lat)
    rng = np.random.default_rng(3)
    f = L.w[:, None] * (1 + 0.2 * rng.uniform(-1, 1, (L.q, 40)))
    rho, u = O.macroscopic(L, f, np.float64)
    feq = O.equilibrium(L, rho, u, np.float64)
    fo = O.bgk(f, feq, 1.7) if coll == "BGK" else O.kbc(L, f, feq, rho, 1.7, np.float64)
    r2, u2 = O.macroscopic(L, fo, np.float64)
    assert np.allclose(r2, rho, rtol=0, atol=1e-14)
    for d in range(L.d):
        assert np.allclose(u2[d] * r2, u[d] * rho, rtol=0, atol=1e-14)


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q27"])
def test_kbc_fixed_point(lat):
    """f = feq is a fixed point of KBC (delta_s = delta_h = 0, gamma = 1/beta)."""
    L = O.Lattice(lat)
    n = 6
    rho = np.linspace(0.9, 1.1, n)
    u = [np.linspace(-0.05, 0.05, n)] * L.d
    feq = O.equilibrium(L, rho, u, np.float64)
    assert np.allclose(O.kbc(L, feq, feq, rho, 1.9, np.float64), feq, atol=1e-16)


@pytest.mark.parametrize("lat", LATS)
def test_zouhe_velocity_known_answer(lat):
    """Zou-He velocity inlet at x = 0: the repaired populations carry the prescribed
    normal velocity and rho = fsum / (1 - u_n) (bc_zouhe.py:292-312)."""
    L = O.Lattice(lat)
    rng = np.random.default_rng(5)
    n = 30
    f = L.w[:, None] * (1 + 0.05 * rng.uniform(-1, 1, (L.q, n)))
    miss = np.zeros((L.q, n), dtype=bool)
    miss[L.c[0] == 1] = True  # pull source x - c is outside for c_x = +1
    v = 0.04
    out = O.zouhe_like(L, f.copy(), miss, np.full(n, v), "zouhe_velocity", np.float64)
    rho, u = O.macroscopic(L, out, np.float64)
    fsum = O.bc_fsum(L, f, miss, np.float64)
    assert np.allclose(rho, fsum / (1 - v), rtol=1e-13)
    assert np.allclose(u[0], v, rtol=1e-12)


@pytest.mark.parametrize("lat", LATS)
def test_zouhe_pressure_known_answer(lat):
    """Pressure outlet at x = nx-1: repaired populations carry the prescribed density."""
    L = O.Lattice(lat)
    rng = np.random.default_rng(6)
    n = 30
    f = L.w[:, None] * (1 + 0.05 * rng.uniform(-1, 1, (L.q, n)))
    miss = np.zeros((L.q, n), dtype=bool)
    miss[L.c[0] == -1] = True
    out = O.zouhe_like(L, f.copy(), miss, np.full(n, 1.02), "zouhe_pressure", np.float64)
    rho, _ = O.macroscopic(L, out, np.float64)
    assert np.allclose(rho, 1.02, rtol=1e-13)


@pytest.mark.parametrize("lat", LATS)
def test_periodic_mass_conservation(lat):
    L = O.Lattice(lat)
    shape = shape_for(lat, 9)
    st = O.Store("f64", L)
    rng = np.random.default_rng(8)
    f0 = L.w.reshape((-1,) + (1,) * 3) * (1 + 0.05 * rng.uniform(-1, 1, (L.q,) + s3(shape)))
    bcm, miss = O.masker(L, shape, [])
    m0 = f0.sum()
    a, _ = O.run(L, st, f0, f0.copy(), bcm, miss, 1.5, [], 6)
    assert abs(a.sum() - m0) < 1e-11 * m0


def test_shifted_storage_roundtrip():
    L = O.Lattice("D3Q19")
    rng = np.random.default_rng(9)
    f = (L.w[:, None] * (1 + 0.01 * rng.uniform(-1, 1, (L.q, 1000)))).astype(np.float32)
    for kind, tol in (("f16s", 2e-6), ("bf16s", 4e-5), ("f16", 2e-4)):
        st = O.Store(kind, L)
        back = st.decode(st.encode(f, np.float32), np.float32)
        assert np.max(np.abs(back - f)) < tol, kind


def test_bf16_rounding_is_nearest_even():
    # bf16 keeps 7 mantissa bits: one ulp at 1.0 is 2**-7
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, 1.0 + 2**-9, 1.0 + 3 * 2**-8, -2.5, np.inf], dtype=np.float32)
    back = O._bf16_to_f32(O._bf16_round(x))
    assert back[0] == 1.0
    assert back[1] == 1.0  # exact tie, rounds to the even mantissa (down)
    assert back[2] == np.float32(1.0 + 2**-7)  # above the tie, up
    assert back[3] == 1.0  # below the tie, down
    assert back[4] == np.float32(1.0 + 2**-6)  # exact tie, rounds to the even mantissa (up)
    assert back[5] == -2.5
    assert np.isinf(back[6])


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19"])
def test_fp32_oracle_tracks_fp64(lat):
    L = O.Lattice(lat)
    shape = shape_for(lat, 10)
    rng = np.random.default_rng(10)
    f64 = L.w.reshape((-1,) + (1,) * 3) * (1 + 0.05 * rng.uniform(-1, 1, (L.q,) + s3(shape)))
    nob = np.array([[i, shape[1] - 1] + ([shape[2] // 2] if len(shape) == 3 else []) for i in range(1, shape[0] - 1)]).T
    bcs = [O.BC("equilibrium", 1, nob, rho=1.0, u=(0.05, 0, 0))]
    bcm, miss = O.masker(L, shape, bcs)
    a64, _ = O.run(L, O.Store("f64", L), f64, f64.copy(), bcm, miss, 1.6, bcs, 10)
    f32 = f64.astype(np.float32)
    a32, _ = O.run(L, O.Store("f32", L), f32, f32.copy(), bcm, miss, 1.6, bcs, 10, T=np.float32)
    assert np.max(np.abs(a32 - a64)) < 2e-6


@pytest.mark.parametrize("lat", LATS)
def test_bgk_pair_form_equals_bgk_to_rounding(lat):
    """The pair form rearranges macroscopic + equilibrium + BGK; in FP64 it agrees
    with XLB's operation order to rounding."""
    L = O.Lattice(lat)
    rng = np.random.default_rng(11)
    f = L.w[:, None] * (1 + 0.2 * rng.uniform(-1, 1, (L.q, 200)))
    rho, u = O.macroscopic(L, f, np.float64)
    want = O.bgk(f, O.equilibrium(L, rho, u, np.float64), 1.7)
    got = O.bgk_pair(L, f, 1.7, np.float64)
    assert np.max(np.abs(got - want)) < 1e-15


def test_fma32_is_correctly_rounded():
    """The oracle's float32 fused multiply-add (used by the pair-form BGK under FP32
    compute) against exact rational arithmetic, including the double-rounding case
    where the float64 sum lands exactly on a float32 midpoint."""
    from fractions import Fraction

    def exact(a, b, c):
        v = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
        lo = np.float32(float(v))
        cands = [np.nextafter(lo, np.float32(-np.inf)), lo, np.nextafter(lo, np.float32(np.inf))]
        return min(cands, key=lambda x: (abs(Fraction(float(x)) - v), int(np.float32(x).view(np.uint32)) & 1))

    # float64 rounds a*b + c up onto the midpoint of 1+2^-23 and 1+2^-22; the exact value is below it
    a = np.float32(2.0**-12 * (1 + 2.0**-23))
    b = np.float32(2.0**-12 * (1 - 2.0**-23))
    c = np.float32(1 + 2.0**-23)
    assert O.fma32(a, b, c) == np.float32(1 + 2.0**-23)
    assert np.float32(np.float64(a) * np.float64(b) + np.float64(c)) != np.float32(1 + 2.0**-23)
    rng = np.random.default_rng(3)
    x, y, z = (rng.standard_normal(500).astype(np.float32) for _ in range(3))
    got = O.fma32(x, y, z)
    assert all(got[i] == exact(x[i], y[i], z[i]) for i in range(500))
    got = O.fma32(x, y, (-(x * y)).astype(np.float32))
    assert all(got[i] == exact(x[i], y[i], -(x[i] * y[i])) for i in range(500))
