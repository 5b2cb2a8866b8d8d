"""CPU restatement of XLB's fused stepper -- TEST INFRASTRUCTURE ONLY.

This module is the oracle that the CUDA path is checked against.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import it, and only as the checker.  Nothing in ``xlb_gb300`` imports it.

It restates, in numpy, the per-cell semantics of XLB's Warp stepper
(xlb/operator/stepper/nse_stepper.py:344-382), vectorised over cells but with
every floating-point operation in the same order as the Warp functionals:

* pull streaming with a one-cell periodic wrap      stream.py:59-82
* streaming-step BCs (f_pre = own-cell f_0)         nse_stepper.py:363-367
* rho / u                                           zero_moment.py:22-27, first_moment.py:25-38
* quadratic equilibrium                             quadratic_equilibrium.py:35-60
* BGK                                               bgk.py:30-34
* KBC (D2Q9, D3Q27)                                 kbc.py:192-296, second_moment.py:68-78
* collision-step BCs + extrapolation aux data       nse_stepper.py:374, bc_extrapolation_outflow.py:390-415
* aux recovery into f_0                             nse_stepper.py:318-342
* store cast                                        nse_stepper.py:379-381

Arithmetic runs in the compute dtype ``T`` (np.float64 or np.float32); numpy
applies IEEE add/sub/mul/div per element with no fused multiply-add, so with
the same operation order the CUDA kernels (built with --fmad=false) reproduce
these results bit for bit.

Two places where XLB's Warp kernel is racy are given one deterministic meaning
here, and the CUDA path implements the same meaning:

1. Aux recovery (nse_stepper.py:338-342) writes f_0 while other threads pull
   from f_0.  By default (``recovery="after"``) recovery happens after every
   pull of the step; ``recovery="before"`` gives the other outcome, where other
   cells' reads see the recovered slots (what a launch gives when the boundary
   cells run first, and what XLB's source gives when run sequentially in cell
   order for an inlet at x = 0).
2. The masker (indices_boundary_masker.py:144-156) writes bc_mask from many
   threads; here boundary conditions are applied in list order, later wins.

The extrapolation-outflow neighbour read (bc_extrapolation_outflow.py:409-413)
has no bounds check in XLB; here its index wraps like the stream does, which
changes nothing for in-range reads.
"""

import itertools

import numpy as np

# ----------------------------------------------------------------------------
# Lattices (xlb/velocity_set/*.py)
# ----------------------------------------------------------------------------


class Lattice:
    def __init__(self, name):
        if name == "D2Q9":
            cx = [0, 0, 0, 1, -1, 1, -1, 1, -1]
            cy = [0, 1, -1, 0, 1, -1, 0, 1, -1]
            c = np.array([cx, cy])
            w = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 9, 1 / 36, 1 / 36])
        elif name == "D3Q19":
            c = np.array([v for v in itertools.product([0, -1, 1], repeat=3) if sum(map(abs, v)) <= 2]).T
            w = np.array([{0: 1 / 3, 1: 1 / 18, 2: 1 / 36}[int(np.abs(c[:, i]).sum())] for i in range(19)])
        elif name == "D3Q27":
            c = np.array(list(itertools.product([0, -1, 1], repeat=3))).T
            w = np.array([{0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}[int(np.abs(c[:, i]).sum())] for i in range(27)])
        else:
            raise ValueError(name)
        self.name = name
        self.c = c.astype(np.int64)
        self.d, self.q = self.c.shape
        self.w = w
        cols = [tuple(v) for v in self.c.T.tolist()]
        self.opp = np.array([cols.index(tuple(-x for x in v)) for v in cols])
        nt = self.d * (self.d + 1) // 2
        cc = np.zeros((self.q, nt))
        k = 0
        for a in range(self.d):
            for b in range(a, self.d):
                cc[:, k] = self.c[a] * self.c[b]
                k += 1
        self.cc = cc
        qi = cc.copy()
        diag, off = ((0, 3, 5), (1, 2, 4)) if self.d == 3 else ((0, 2), (1,))
        qi[:, diag] += -1.0 / 3.0
        qi[:, off] *= 2.0
        self.qi = qi


# ----------------------------------------------------------------------------
# Storage forms
# ----------------------------------------------------------------------------


def _bf16_round(x32):
    """float32 -> bfloat16 bits (uint16), round to nearest even."""
    b = np.ascontiguousarray(x32, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounded = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    nan = np.isnan(x32)
    out = rounded.astype(np.uint16)
    out[nan] = 0x7FC0
    return out


def _bf16_to_f32(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


# The FP16 shifted form stores (f - w_l) * 2^14: the scale keeps deviations
# down to about 4e-9 in FP16's normal range (its smallest normal is 6.1e-5), where
# the unscaled form would fall into subnormals with 6e-8 absolute resolution.
# A power of two scales exactly, so the only roundings are f - w_l in FP32 and
# the conversion to FP16.
F16S_SCALE = np.float32(2.0**14)
F16S_INV_SCALE = np.float32(2.0**-14)


class Store:
    """How populations live in memory: 'f64', 'f32', 'f16' (raw) or the shifted
    'f16s' / 'bf16s' forms (stored value = (f - w_l) * 2^14 in FP16, f - w_l in
    BF16)."""

    def __init__(self, kind, lattice):
        self.kind = kind
        self.lat = lattice
        self.shifted = kind in ("f16s", "bf16s")

    @property
    def np_dtype(self):
        return {"f64": np.float64, "f32": np.float32, "f16": np.float16, "f16s": np.float16, "bf16s": np.uint16}[self.kind]

    def _w(self, T, ndim):
        return self.lat.w.astype(T).reshape((-1,) + (1,) * (ndim - 1))

    def encode(self, f, T):
        """compute-dtype populations (q, ...) -> stored array."""
        f = np.asarray(f, dtype=T)
        if self.kind in ("f64", "f32", "f16"):
            return f.astype(self.np_dtype)
        dev = (f - self._w(T, f.ndim)).astype(np.float32)
        if self.kind == "f16s":
            return (dev * F16S_SCALE).astype(np.float16)
        return _bf16_round(dev)

    def decode(self, s, T):
        """stored array (q, ...) -> compute-dtype populations."""
        if self.kind in ("f64", "f32", "f16"):
            return s.astype(T)
        raw = s.astype(np.float32) * F16S_INV_SCALE if self.kind == "f16s" else _bf16_to_f32(s)
        return raw.astype(T) + self._w(T, s.ndim)

    def encode_raw(self, x, T):
        """A non-population value (boundary aux data) stored without shift."""
        x = np.asarray(x, dtype=T)
        if self.kind == "bf16s":
            return _bf16_round(x.astype(np.float32))
        return x.astype(self.np_dtype)

    def decode_raw(self, s, T):
        if self.kind == "bf16s":
            return _bf16_to_f32(np.asarray(s)).astype(T)
        return np.asarray(s).astype(T)

    # The populations as the deviation-space collision (code 3) sees them:
    # g = scale * (f - w_l), the stored value itself for the shifted forms.
    @property
    def scale(self):
        return F16S_SCALE if self.kind == "f16s" else np.float32(1.0)

    def deviation(self, s):
        """stored array -> float32 g: the stored value of the shifted forms
        (exact), f - w_l for FP32 (exact while w_l/2 <= f <= 2 w_l)."""
        if self.kind == "f32":
            return s.astype(np.float32) - self._w(np.float32, s.ndim)
        return s.astype(np.float32) if self.kind == "f16s" else _bf16_to_f32(s)

    def encode_deviation(self, g):
        """float32 g -> stored array (round to nearest even; FP32 stores w_l + g)."""
        g = np.asarray(g, dtype=np.float32)
        if self.kind == "f32":
            return (g + self._w(np.float32, g.ndim)).astype(np.float32)
        return g.astype(np.float16) if self.kind == "f16s" else _bf16_round(g)



# ----------------------------------------------------------------------------
# Boundary-condition descriptions
# ----------------------------------------------------------------------------

STREAMING_KINDS = ("halfway_bb", "equilibrium", "zouhe_velocity", "zouhe_pressure", "regularized_velocity", "regularized_pressure", "extrapolation")
RECOVERY_KINDS = ("zouhe_velocity", "zouhe_pressure", "regularized_velocity", "regularized_pressure")
PADDING_KINDS = ("halfway_bb",) + RECOVERY_KINDS


class BC:
    """kind, id, indices (d, n) and optional parameters.

    kinds: fullway_bb, halfway_bb, equilibrium, zouhe_velocity, zouhe_pressure,
    regularized_velocity, regularized_pressure, extrapolation.
    """

    def __init__(self, kind, bc_id, indices, rho=1.0, u=(0.0, 0.0, 0.0), value=None, profile=None):
        self.kind = kind
        self.id = int(bc_id)
        self.indices = np.asarray(indices, dtype=np.int64)
        self.rho = rho
        self.u = tuple(u)
        self.value = value  # constant prescribed value (ZouHe / Regularized)
        self.profile = profile  # callable(idx3 (3, n) int array) -> (n,) values

    @property
    def needs_padding(self):
        return self.kind in PADDING_KINDS


def _shape3(shape):
    return tuple(shape) if len(shape) == 3 else (shape[0], shape[1], 1)


def check_bc_overlaps(bcs, d):
    """Duplicate indices raise, as XLB's Warp path does (check_boundary_overlaps.py:5-24)."""
    allidx = []
    for bc in bcs:
        idx = np.asarray(bc.indices)[:d]
        if np.unique(idx, axis=-1).shape[-1] != idx.shape[-1]:
            raise ValueError(f"Boundary condition {bc.kind} has duplicate indices!")
        allidx.append(idx)
    if allidx:
        cat = np.concatenate(allidx, axis=1)
        if np.unique(cat, axis=-1).shape[-1] != cat.shape[-1]:
            raise ValueError("Boundary condition list containes duplicate indices!")


def masker(lat, shape, bcs):
    """bc_mask (1, nx, ny, nz) uint8 and missing_mask (q, nx, ny, nz) bool.

    Follows the Warp IndicesBoundaryMasker kernel (indices_boundary_masker.py:114-156
    and its host side :160-224): every index gets its BC id; a direction whose pull
    source is outside the domain is missing; for padding BCs whose index lies in
    the domain interior (:29-40), each in-bounds direction marks the push
    neighbour x + c_l as missing in l and gives it the BC id (l = 0 marks the
    cell itself).  BCs are applied in list order.
    """
    s3 = _shape3(shape)
    d = lat.d
    bc_mask = np.zeros((1,) + s3, dtype=np.uint8)
    missing = np.zeros((lat.q,) + s3, dtype=bool)
    shp = np.array(s3)
    for bc in bcs:
        idx = np.asarray(bc.indices, dtype=np.int64)
        if idx.shape[0] == 2:
            idx = np.vstack([idx, np.zeros(idx.shape[1], dtype=np.int64)])
        inb = np.all((idx >= 0) & (idx < shp[:, None]), axis=0)
        idx = idx[:, inb]
        if bc.needs_padding:
            interior = np.all((idx[:d] > 0) & (idx[:d] < shp[:d, None] - 1), axis=0)
        else:
            interior = np.zeros(idx.shape[1], dtype=bool)
        bc_mask[0, idx[0], idx[1], idx[2]] = bc.id
        for l in range(lat.q):
            c3 = np.zeros(3, dtype=np.int64)
            c3[:d] = lat.c[:, l]
            pull = idx - c3[:, None]
            pull[d:] = 0  # pull_index[d:] keeps its zero initialisation (:137-141)
            pin = np.all((pull >= 0) & (pull < shp[:, None]), axis=0)
            out = ~pin
            missing[l, idx[0, out], idx[1, out], idx[2, out]] = True
            sel = pin & interior
            push = idx[:, sel] + c3[:, None]
            missing[l, push[0], push[1], push[2]] = True
            bc_mask[0, push[0], push[1], push[2]] = bc.id
    return bc_mask, missing


def cell_indices(bc_mask, bc_id):
    return np.array(np.nonzero(bc_mask[0] == bc_id))


def aux_init(lat, store, f1, bc_mask, missing, bcs, T):
    """Write prescribed values into f_1[0] at ZouHe / Regularized cells
    (boundary_condition.py:130-159; num_of_aux_data = 1 so only slot 0 is used,
    bc_zouhe.py:110).  Returns a new f_1."""
    f1 = f1.copy()
    for bc in bcs:
        if bc.kind not in RECOVERY_KINDS:
            continue
        cells = cell_indices(bc_mask, bc.id)
        if bc.profile is not None:
            vals = np.asarray(bc.profile(cells), dtype=np.float64).reshape(-1)
        else:
            vals = np.full(cells.shape[1], bc.value, dtype=np.float64)
        f1[0, cells[0], cells[1], cells[2]] = store.encode_raw(vals, T)
    return f1


# ----------------------------------------------------------------------------
# Per-cell functionals, vectorised over a set of cells.  Arrays are (q, n).
# ----------------------------------------------------------------------------


def pull(lat, f):
    """f_ps[l](x) = f[l](x - c_l) with a one-cell periodic wrap (stream.py:64-82)."""
    out = np.empty_like(f)
    for l in range(lat.q):
        shift = tuple(int(v) for v in lat.c[:, l])
        out[l] = np.roll(f[l], shift, axis=tuple(range(lat.d)))
    return out


def macroscopic(lat, f, T):
    rho = T(0.0) + f[0]
    for l in range(1, lat.q):
        rho = rho + f[l]
    u = []
    for d in range(lat.d):
        acc = np.zeros_like(rho)
        for l in range(lat.q):
            if lat.c[d, l] == 1:
                acc = acc + f[l]
            elif lat.c[d, l] == -1:
                acc = acc - f[l]
        u.append(acc / rho)
    return rho, u


def equilibrium(lat, rho, u, T):
    """feq_l = rho w_l (1 + cu (1 + cu/2) - 1.5 |u|^2), cu = 3 c_l.u (quadratic_equilibrium.py:340-354)."""
    w = lat.w.astype(T)
    usq = u[0] * u[0]
    for d in range(1, lat.d):
        usq = usq + u[d] * u[d]
    usqr = T(1.5) * usq
    feq = []
    for l in range(lat.q):
        cu = np.zeros_like(rho)
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                cu = cu + u[d]
            elif lat.c[d, l] == -1:
                cu = cu - u[d]
        cu = cu * T(3.0)
        feq.append(rho * w[l] * (T(1.0) + cu * (T(1.0) + T(0.5) * cu) - usqr))
    return np.stack(feq)


def bgk(f, feq, omega_t):
    return f - omega_t * (f - feq)


def fma32(a, b, c):
    """Correctly rounded float32 a * b + c (what the CUDA __fmaf_rn and C fmaf give).

    The float64 product of two float32 values is exact; the float64 sum p + c
    rounds once, and TwoSum recovers its error e exactly.  Rounding the float64
    sum to float32 is then correct except when it lands exactly on the midpoint
    between two float32 neighbours while e != 0: the exact value then lies on
    the side given by the sign of e."""
    a64 = np.asarray(a, dtype=np.float32).astype(np.float64)
    b64 = np.asarray(b, dtype=np.float32).astype(np.float64)
    c64 = np.asarray(c, dtype=np.float32).astype(np.float64)
    p = a64 * b64
    s = p + c64
    bb = s - p
    e = (p - (s - bb)) + (c64 - bb)
    r = s.astype(np.float32)
    r64 = r.astype(np.float64)
    # the float32 neighbour of r on the side of s, and the midpoint between them
    toward = np.where(s > r64, np.float32(np.inf), np.float32(-np.inf)).astype(np.float32)
    n = np.nextafter(r, toward)
    mid = (r64 + n.astype(np.float64)) * 0.5
    tie = (s == mid) & (s != r64) & (e != 0)
    # at a tie, RN picked r or n by parity; the exact value is beyond the midpoint on e's side
    up = np.where(r64 > n.astype(np.float64), r, n)
    down = np.where(r64 > n.astype(np.float64), n, r)
    fixed = np.where(e > 0, up, down)
    return np.where(tie, fixed, r).astype(np.float32)


def bgk_pair(lat, f, omega_t, T):
    """BGK with macroscopic and equilibrium arranged over opposite-direction pairs
    (collision code 2; no XLB counterpart).  Same equations as macroscopic +
    equilibrium + bgk; the operation order below is the CUDA path's, including
    its fused multiply-adds under FP32 compute (fma32)."""
    pairs = [l for l in range(1, lat.q) if l < lat.opp[l]]
    rho = f[0].copy()
    j = [np.zeros_like(rho) for _ in range(lat.d)]
    for l in pairs:
        o = lat.opp[l]
        sig = f[l] + f[o]
        dif = f[l] - f[o]
        rho = rho + sig
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                j[d] = j[d] + dif
            elif lat.c[d, l] == -1:
                j[d] = j[d] - dif
    inv = T(1.0) / rho
    u = [jd * inv for jd in j]
    fused = T == np.float32  # FP32 compute fuses multiply-adds, FP64 keeps two roundings
    usq = u[0] * u[0]
    for d in range(1, lat.d):
        usq = fma32(u[d], u[d], usq) if fused else usq + u[d] * u[d]
    base = fma32(T(-1.5), usq, T(1.0)) if fused else T(1.0) - T(1.5) * usq
    omf = T(1.0) - omega_t
    orho = omega_t * rho
    w = lat.w.astype(T)
    fo = np.empty_like(f)
    fo[0] = fma32(omf, f[0], orho * w[0] * base) if fused else omf * f[0] + orho * w[0] * base
    for l in pairs:
        o = lat.opp[l]
        cu = np.zeros_like(rho)
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                cu = cu + u[d]
            elif lat.c[d, l] == -1:
                cu = cu - u[d]
        t = T(3.0) * cu
        ow = orho * w[l]
        if fused:
            e = fma32(T(4.5) * cu, cu, base)
            fo[l] = fma32(omf, f[l], ow * (e + t))
            fo[o] = fma32(omf, f[o], ow * (e - t))
        else:
            e = base + T(4.5) * (cu * cu)
            fo[l] = omf * f[l] + ow * (e + t)
            fo[o] = omf * f[o] + ow * (e - t)
    return fo


def bgk_shifted(lat, g, omega_t, scale):
    """BGK on the stored deviations g = scale (f - w_l) of the shifted stores
    (collision code 3; no XLB counterpart).  Same equations as macroscopic +
    equilibrium + bgk (bgk.py:30-34, quadratic_equilibrium.py:35-60) in pair
    form, rewritten for g:
      rho = 1 + G/scale, v = 3u = 3 J/(scale rho), base = 1 - |v|^2/6,
      r = rho base - 1 = (G/scale) base - |v|^2/6 (no cancellation),
      per weight class k: A = omega scale w_k (two floats hi + lo: a rounded A
        is a systematic error of the class that breaks momentum conservation),
        A rho and C = A r each rounded once,
      per pair (l, o) with t = c_l.v: R = C + (A rho / 2) t^2,
      g_out_l = (1 - omega) g_l + (A rho t + R), g_out_o = (1 - omega) g_o + (-A rho t + R).
    FP32 only; the operation order (and every fused multiply-add, fma32) is the
    CUDA path's."""
    f32 = np.float32
    S = f32(scale)
    K = f32(1.0) / S
    pairs = [l for l in range(1, lat.q) if l < lat.opp[l]]
    G = g[0].copy()
    J = [np.zeros_like(G) for _ in range(lat.d)]
    for l in pairs:
        o = lat.opp[l]
        sig = g[l] + g[o]
        dif = g[l] - g[o]
        G = G + sig
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                J[d] = J[d] + dif
            elif lat.c[d, l] == -1:
                J[d] = J[d] - dif
    rho = fma32(K, G, f32(1.0))
    inv = f32(1.0) / rho
    k3 = f32(3.0) * (K * inv)
    v = [Jd * k3 for Jd in J]
    vsq = v[0] * v[0]
    for d in range(1, lat.d):
        vsq = fma32(v[d], v[d], vsq)
    bm1 = (f32(-1.0) / f32(6.0)) * vsq
    base = f32(1.0) + bm1
    r = fma32(K * G, base, bm1)  # rho base - 1 without cancellation
    omf = f32(1.0) - f32(omega_t)
    norm1 = np.abs(lat.c).sum(axis=0)
    Ar, Arh, C = {}, {}, {}
    om = f32(omega_t)
    for k in sorted(set(norm1.tolist())):
        # A = omega S w_k carried as hi + lo (S w_k split into two floats in float64)
        sw = float(S) * float(lat.w[int(np.argmax(norm1 == k))])
        whi = f32(sw)
        wlo = f32(sw - float(whi))
        ahi = om * whi
        alo = fma32(om, whi, -ahi) + om * wlo
        Ar[k] = fma32(ahi, rho, alo * rho)
        Arh[k] = f32(0.5) * Ar[k]
        C[k] = fma32(ahi, r, alo * r)
    go = np.empty_like(g)
    go[0] = fma32(omf, g[0], C[0])
    for l in pairs:
        o = lat.opp[l]
        k = int(norm1[l])
        t = None
        for d in range(lat.d):
            if lat.c[d, l] != 0:
                x = v[d] if lat.c[d, l] == 1 else -v[d]
                t = x if t is None else t + x
        q = Arh[k] * t
        R = fma32(q, t, C[k])
        go[l] = fma32(omf, g[l], fma32(Ar[k], t, R))
        go[o] = fma32(omf, g[o], fma32(-Ar[k], t, R))
    return go


def second_moment(lat, fneq, T):
    nt = lat.d * (lat.d + 1) // 2
    pi = []
    for t in range(nt):
        acc = np.zeros_like(fneq[0])
        for q in range(lat.q):
            cc = lat.cc[q, t]
            if cc == 1:
                acc = acc + fneq[q]
            elif cc == -1:
                acc = acc - fneq[q]
        pi.append(acc)
    return pi


def kbc(lat, f, feq, rho, omega_t, T):
    """Entropic KBC collision, D2Q9 and D3Q27 only (kbc.py:192-296)."""
    fneq = f - feq
    pi = second_moment(lat, fneq, T)
    s = np.zeros_like(f)
    two, four, six = T(2.0), T(4.0), T(6.0)
    if lat.name == "D3Q27":
        nxz = pi[0] - pi[5]
        nyz = pi[3] - pi[5]
        a = (two * nxz - nyz) / six
        b = (-nxz + two * nyz) / six
        cz = (-nxz - nyz) / six
        s[9], s[18], s[3], s[6], s[1], s[2] = a, a, b, b, cz, cz
        p1, p2, p4 = pi[1] / four, pi[2] / four, pi[4] / four
        m1, m2, m4 = -pi[1] / four, -pi[2] / four, -pi[4] / four
        s[12], s[24], s[21], s[15] = p1, p1, m1, m1
        s[10], s[20], s[19], s[11] = p2, p2, m2, m2
        s[8], s[4], s[7], s[5] = p4, p4, m4, m4
        delta_s = s * rho
    elif lat.name == "D2Q9":
        n = pi[0] - pi[2]
        s[3], s[6], s[2], s[1] = n, n, -n, -n
        s[8], s[4], s[5], s[7] = pi[1], -pi[1], -pi[1], pi[1]
        delta_s = s * rho / four
    else:
        raise NotImplementedError(f"KBC is not defined for {lat.name}")
    beta = T(0.5) * omega_t
    inv_beta = T(1.0) / beta
    delta_h = fneq - delta_s
    temp = delta_h / feq
    sp1 = np.zeros_like(rho)
    sp2 = np.zeros_like(rho)
    for l in range(lat.q):
        sp1 = sp1 + temp[l] * delta_s[l]
        sp2 = sp2 + temp[l] * delta_h[l]
    gamma = inv_beta - (two - inv_beta) * sp1 / (T(1e-32) + sp2)
    return f - beta * (two * delta_s + gamma * delta_h)


def normals_float(lat, miss, T):
    """-c of the first missing direction with |c|_1 = 1 (helper_functions_bc.py:250-261).
    Cells with no such direction get a zero normal."""
    n = miss.shape[1]
    found = np.zeros(n, dtype=bool)
    nv = np.zeros((lat.d, n), dtype=np.int64)
    for l in range(lat.q):
        if np.abs(lat.c[:, l]).sum() != 1:
            continue
        take = miss[l] & ~found
        nv[:, take] = -lat.c[:, l][:, None]
        found |= take
    return nv


def bc_fsum(lat, f, miss, T):
    """Known (x2) plus middle populations (helper_functions_bc.py:236-248)."""
    known = np.zeros_like(f[0])
    middle = np.zeros_like(f[0])
    for l in range(lat.q):
        k = miss[lat.opp[l]]
        m = (~k) & (~miss[l])
        known = np.where(k, known + T(2.0) * f[l], known)
        middle = np.where(m, middle + f[l], middle)
    return known + middle


def bounceback_noneq(lat, f, feq, miss):
    f = f.copy()
    for l in range(lat.q):
        o = lat.opp[l]
        f[l] = np.where(miss[l], f[o] + feq[l] - feq[o], f[l])
    return f


def regularize(lat, f, feq, T):
    """f = feq + 4.5 w_l (qi_l : Pi(f - feq)) (helper_functions_bc.py:274-297)."""
    pi = second_moment(lat, f - feq, T)
    qi = lat.qi.astype(T)
    w = lat.w.astype(T)
    out = np.empty_like(f)
    nt = len(pi)
    for l in range(lat.q):
        acc = np.zeros_like(f[0])
        for t in range(nt):
            if lat.qi[l, t] != 0.0:
                acc = acc + qi[l, t] * pi[t]
        out[l] = feq[l] + T(4.5) * w[l] * acc
    return out


def zouhe_like(lat, f, miss, aux, kind, T):
    """ZouHe / Regularized, velocity or pressure (bc_zouhe.py:279-343, bc_regularized.py:134-202)."""
    nv = normals_float(lat, miss, T).astype(T)
    fsum = bc_fsum(lat, f, miss, T)
    if kind.endswith("velocity"):
        u = [(-aux) * nv[d] for d in range(lat.d)]
        unormal = np.zeros_like(fsum)
        for d in range(lat.d):
            unormal = unormal + u[d] * nv[d]
        rho = fsum / (T(1.0) + unormal)
    else:
        rho = aux
        unormal = T(-1.0) + fsum / rho
        u = [unormal * nv[d] for d in range(lat.d)]
    feq = equilibrium(lat, rho, u, T)
    out = bounceback_noneq(lat, f, feq, miss)
    if kind.startswith("regularized"):
        out = regularize(lat, out, feq, T)
    return out


def equilibrium_dev(lat, drho, u, scale):
    """scale (feq_l - w_l) from rho - 1 and u, without cancellation against 1
    or w_l (collision code 3; the CUDA path's equilibrium_dev, FP32):
    rho e_l - 1 = drho e_l + (e_l - 1), e_l - 1 = t + t^2/2 - 1.5|u|^2, t = 3 c_l.u."""
    f32 = np.float32
    usq = u[0] * u[0]
    for d in range(1, lat.d):
        usq = fma32(u[d], u[d], usq)
    b = f32(-1.5) * usq
    w = lat.w.astype(f32)
    geq = []
    for l in range(lat.q):
        cu = np.zeros_like(usq)
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                cu = cu + u[d]
            elif lat.c[d, l] == -1:
                cu = cu - u[d]
        t = f32(3.0) * cu
        em1 = fma32(f32(0.5) * t, t, t + b)
        e = f32(1.0) + em1
        geq.append((f32(scale) * w[l]) * fma32(drho, e, em1))
    return np.stack(geq)


def zouhe_like_dev(lat, g, miss, aux, kind, scale):
    """ZouHe / Regularized on deviations g = scale (f - w) (collision code 3,
    FP32; the CUDA path's zouhe_like_dev).  XLB's fsum (helper_functions_bc.py:
    236-248) is 1 + dW + G/scale with G the same selection summed over g and dW
    the weights of directions missing together with their opposite; rho - 1 and
    u follow from it as in bc_zouhe.py:279-343 without forming rho near 1."""
    f32 = np.float32
    K = f32(1.0) / f32(scale)
    nv = normals_float(lat, miss, f32).astype(f32)
    w = lat.w.astype(f32)
    G = np.zeros_like(g[0])
    dW = np.zeros_like(g[0])
    for l in range(lat.q):
        k = miss[lat.opp[l]]
        m = (~k) & (~miss[l])
        G = np.where(k, G + f32(2.0) * g[l], G)
        G = np.where(m, G + g[l], G)
        dW = np.where(k & miss[l], dW + w[l], dW)
    fs1 = fma32(K, G, dW)
    if kind.endswith("velocity"):
        u = [(-aux) * nv[d] for d in range(lat.d)]
        unormal = np.zeros_like(fs1)
        for d in range(lat.d):
            unormal = unormal + u[d] * nv[d]
        drho = (fs1 - unormal) / (f32(1.0) + unormal)
    else:
        drho = aux - f32(1.0)
        unormal = (fs1 - drho) / aux
        u = [unormal * nv[d] for d in range(lat.d)]
    geq = equilibrium_dev(lat, drho, u, scale)
    g = bounceback_noneq(lat, g, geq, miss)
    if kind.startswith("regularized"):
        g = regularize(lat, g, geq, f32)
    return g


def extrapolation_cs(T):
    """cs = 1/sqrt(3) as XLB builds it: compute_dtype(1.0 / wp.sqrt(3.0))
    (bc_extrapolation_outflow.py:353); Warp evaluates wp.sqrt(3.0) at Python
    scope in float32."""
    return T(1.0 / float(np.sqrt(np.float32(3.0))))


# ----------------------------------------------------------------------------
# The step
# ----------------------------------------------------------------------------


def _recovered(lat, f0, f1, bc_mask, missing, bcs, with_slot0=True):
    """f0 with the aux-recovery writes of nse_stepper.py:318-342 applied."""
    out = f0.copy()
    for bc in bcs:
        if bc.kind not in RECOVERY_KINDS:
            continue
        m = bc_mask[0] == bc.id
        if with_slot0:
            out[0][m] = f1[0][m]
        for l in range(1, lat.q):
            mm = m & missing[l]
            o = lat.opp[l]
            out[o][mm] = f1[o][mm]
    return out


def step(lat, store, f0, f1, bc_mask, missing, omega, bcs, collision="BGK", T=np.float64, recovery="after",
         timestep=0):
    """One fused step.  Returns (f0_new, f1_new) as stored arrays.

    f0_new differs from f0 only where aux recovery wrote it
    (nse_stepper.py:318-342); f1_new holds the post-collision state except at
    cells with id 255, which the kernel skips (:356-358).

    ``recovery`` resolves XLB's race between the recovery writes into f0 and
    other cells' reads of f0: "after" (the CUDA path's order) lets every read
    of the step see the pre-step f0; "before" lets reads of *other* cells see
    the recovered slots, which is what a launch gives when the ZouHe /
    Regularized cells run before the cells reading them.
    """
    if collision in ("BGK_SHIFTED", "BGK_SHIFTED_SR"):
        return _step_shifted(lat, store, f0, f1, bc_mask, missing, omega, bcs, recovery,
                             stochastic=collision == "BGK_SHIFTED_SR", timestep=timestep)
    shp = f0.shape[1:]
    ids = bc_mask[0]
    f0c = store.decode(f0, T)
    f0r = f0c if recovery == "after" else store.decode(_recovered(lat, f0, f1, bc_mask, missing, bcs, with_slot0=False), T)
    fps = pull(lat, f0r)
    omega_t = T(omega)
    by_id = {bc.id: bc for bc in bcs}

    # streaming-step BCs, f_pre = own-cell f_0, f_post = pulled values
    for bc in bcs:
        if bc.kind not in STREAMING_KINDS:
            continue
        m = ids == bc.id
        if not m.any():
            continue
        fp = fps[:, m]
        miss = missing[:, m]
        own = f0c[:, m]
        if bc.kind in ("halfway_bb", "extrapolation"):
            for l in range(lat.q):
                fp[l] = np.where(miss[l], own[lat.opp[l]], fp[l])
        elif bc.kind == "equilibrium":
            rho_bc = np.full(fp.shape[1], T(bc.rho), dtype=T)
            u_bc = [np.full(fp.shape[1], T(bc.u[d]), dtype=T) for d in range(lat.d)]
            fp = equilibrium(lat, rho_bc, u_bc, T)
        else:
            aux = store.decode_raw(f1[0][m], T)
            fp = zouhe_like(lat, fp, miss, aux, bc.kind, T)
        fps[:, m] = fp

    if collision == "BGK_PAIR":
        fout = bgk_pair(lat, fps, omega_t, T)
    else:
        rho, u = macroscopic(lat, fps, T)
        feq = equilibrium(lat, rho, u, T)
        if collision == "BGK":
            fout = bgk(fps, feq, omega_t)
        elif collision == "KBC":
            fout = kbc(lat, fps, feq, rho, omega_t, T)
        else:
            raise ValueError(collision)

    # collision-step BCs and the extrapolation aux data (nse_stepper.py:286-293)
    for bc in bcs:
        m = ids == bc.id
        if not m.any():
            continue
        if bc.kind == "fullway_bb":
            fout[:, m] = fps[:, m][lat.opp]
        elif bc.kind == "extrapolation":
            cs = extrapolation_cs(T)
            miss = missing[:, m]
            cells = np.array(np.nonzero(m))
            nv = normals_float(lat, miss, T)
            fo = fout[:, m]
            fp = fps[:, m]
            for l in range(lat.q):
                sel = miss[l]
                if not sel.any():
                    continue
                src = cells[:, sel].copy()
                for d in range(lat.d):
                    src[d] = (src[d] - (lat.c[d, l] + nv[d, sel])) % shp[d]
                f_aux = f0r[l][tuple(src)]
                fo[lat.opp[l], sel] = (T(1.0) - cs) * fp[l, sel] + cs * f_aux
            fout[:, m] = fo

    f1_new = store.encode(fout, T)
    skip = ids == 255
    if skip.any():
        f1_new[:, skip] = f1[:, skip]

    return _recovered(lat, f0, f1, bc_mask, missing, bcs), f1_new


def sr_seed(cell, t):
    """Random bits of one cell's stochastic rounding (collision code 4): the
    "lowbias32" integer hash (C. Wellons) of cell * 0x9E3779B1 + t * 0x85EBCA77,
    uint32 arithmetic as the CUDA path's sr_seed."""
    x = np.asarray(cell, dtype=np.uint64).astype(np.uint32) * np.uint32(0x9E3779B1) + np.uint32(
        (int(t) * 0x85EBCA77) & 0xFFFFFFFF)
    x = x ^ (x >> np.uint32(16))
    x = x * np.uint32(0x7FEB352D)
    x = x ^ (x >> np.uint32(15))
    x = x * np.uint32(0x846CA68B)
    return x ^ (x >> np.uint32(16))


def sr_bits(seed, k):
    return seed * np.uint32(((2 * k + 1) * 0x9E3779B9) & 0xFFFFFFFF)


def sr_round_f16(x, r16):
    """Blackwell's cvt.rs to FP16 of float32 x with 16 random bits r16 (the CUDA
    path's sr_pack, pinned on the GPU bit for bit): floor(|x| / ulp + r13 / 2^13)
    ulp with r13 = r16 & 0x1FFF and ulp the FP16 ulp of |x|'s binade (2^-24 below
    2^-14), signed; +-inf from 65536 up.  Returns the FP16 bits."""
    x = np.asarray(x, dtype=np.float32)
    ax = np.abs(x.astype(np.float64))
    e = np.floor(np.log2(np.where(ax > 0, ax, 1.0)))
    ulp = np.where(ax < 2.0**-14, 2.0**-24, 2.0 ** (e - 10))
    v = ax / ulp
    k = np.floor(v)
    q = k + ((v - k) + (np.asarray(r16).astype(np.uint32) & np.uint32(0x1FFF)).astype(np.float64) / 8192.0 >= 1.0)
    val = q * ulp
    with np.errstate(over="ignore"):
        h = np.where(val >= 65536.0, np.inf, val).astype(np.float16)
    h = np.where(np.signbit(x), -h, h).astype(np.float16)
    return h.view(np.uint16)


def sr_round_bf16(x, r16):
    """cvt.rs to BF16: the 16 random bits added to the low half of x's float32
    pattern, then truncated to the upper half.  Returns the BF16 bits."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + (np.asarray(r16).astype(np.uint64) & 0xFFFF)) >> 16).astype(np.uint16)


def encode_stochastic(store, g, timestep):
    """Stored bits of deviations g (q, *shape) with stochastic rounding: pairs of
    directions (2k, 2k + 1) share one 32-bit word of random bits, the lower
    direction its low half (the CUDA path's store with collision code 4)."""
    q = g.shape[0]
    flat = np.asarray(g, dtype=np.float32).reshape(q, -1)
    seed = sr_seed(np.arange(flat.shape[1], dtype=np.uint64), timestep)
    rnd = sr_round_f16 if store.kind == "f16s" else sr_round_bf16
    out = np.empty(flat.shape, dtype=np.uint16)
    for l in range(0, q, 2):
        r = sr_bits(seed, l // 2)
        out[l] = rnd(flat[l], r & np.uint32(0xFFFF))
        if l + 1 < q:
            out[l + 1] = rnd(flat[l + 1], r >> np.uint32(16))
    out = out.reshape(g.shape)
    return out.view(np.float16) if store.kind == "f16s" else out


def _step_shifted(lat, store, f0, f1, bc_mask, missing, omega, bcs, recovery, stochastic=False, timestep=0):
    """step() with collision code 3 (shifted or FP32 stores, FP32): every pulled value,
    streaming-step result and collision output is a deviation g.  The
    bounce-back kinds copy deviations (w_l = w_opp(l)), the extrapolation blend
    is the same linear expression on g, and EquilibriumBC / ZouHe / Regularized
    run on deviations (equilibrium_dev, zouhe_like_dev)."""
    if not (store.shifted or store.kind == "f32"):
        raise ValueError("BGK_SHIFTED needs a shifted or FP32 store")
    T = np.float32
    shp = f0.shape[1:]
    ids = bc_mask[0]
    g0 = store.deviation(f0)
    g0r = g0 if recovery == "after" else store.deviation(_recovered(lat, f0, f1, bc_mask, missing, bcs, with_slot0=False))
    gps = pull(lat, g0r)
    for bc in bcs:
        if bc.kind not in STREAMING_KINDS:
            continue
        m = ids == bc.id
        if not m.any():
            continue
        gp = gps[:, m]
        miss = missing[:, m]
        own = g0[:, m]
        if bc.kind in ("halfway_bb", "extrapolation"):
            for l in range(lat.q):
                gp[l] = np.where(miss[l], own[lat.opp[l]], gp[l])
        elif bc.kind == "equilibrium":
            drho = np.full(gp.shape[1], T(bc.rho - 1.0), dtype=T)
            u_bc = [np.full(gp.shape[1], T(bc.u[d]), dtype=T) for d in range(lat.d)]
            gp = equilibrium_dev(lat, drho, u_bc, store.scale)
        else:
            aux = store.decode_raw(f1[0][m], T)
            gp = zouhe_like_dev(lat, gp, miss, aux, bc.kind, store.scale)
        gps[:, m] = gp

    gout = bgk_shifted(lat, gps, T(omega), store.scale)

    for bc in bcs:
        m = ids == bc.id
        if not m.any():
            continue
        if bc.kind == "fullway_bb":
            gout[:, m] = gps[:, m][lat.opp]
        elif bc.kind == "extrapolation":
            cs = extrapolation_cs(T)
            miss = missing[:, m]
            cells = np.array(np.nonzero(m))
            nv = normals_float(lat, miss, T)
            go = gout[:, m]
            gp = gps[:, m]
            for l in range(lat.q):
                sel = miss[l]
                if not sel.any():
                    continue
                src = cells[:, sel].copy()
                for d in range(lat.d):
                    src[d] = (src[d] - (lat.c[d, l] + nv[d, sel])) % shp[d]
                g_aux = g0r[l][tuple(src)]
                go[lat.opp[l], sel] = (T(1.0) - cs) * gp[l, sel] + cs * g_aux
            gout[:, m] = go

    f1_new = encode_stochastic(store, gout, timestep) if stochastic else store.encode_deviation(gout)
    skip = ids == 255
    if skip.any():
        f1_new[:, skip] = f1[:, skip]
    return _recovered(lat, f0, f1, bc_mask, missing, bcs), f1_new


def run(lat, store, f0, f1, bc_mask, missing, omega, bcs, steps, collision="BGK", T=np.float64, recovery="after",
        timestep0=0):
    """``steps`` steps with the caller-side swap of XLB's examples
    (mlups_3d.py:78-80).  Returns (f_0, f_1) after the final swap: f_0 holds the
    newest state."""
    for k in range(steps):
        f0, f1 = step(lat, store, f0, f1, bc_mask, missing, omega, bcs, collision, T, recovery, timestep0 + k)
        f0, f1 = f1, f0
    return f0, f1


def initial_equilibrium(lat, store, shape, T, rho=1.0, u=None):
    """f = feq(rho=1, u=0) in the store form (initializers.py:5-20)."""
    s3 = _shape3(shape)
    n = int(np.prod(s3))
    rho_a = np.full(n, T(rho), dtype=T)
    u_a = [np.full(n, T(0.0 if u is None else u[d]), dtype=T) for d in range(lat.d)]
    feq = equilibrium(lat, rho_a, u_a, T).reshape((lat.q,) + s3)
    return store.encode(feq, T)


def momentum_transfer(lat, store, f0, bc_mask, missing, bc_id, T=np.float64):
    """Force on a no-slip BC by momentum exchange (momentum_transfer.py:108-160).

    For the no-slip functionals (halfway or fullway bounce-back) the post-stream
    value in a missing direction is f_0[opp l] at the cell, so
    phi_l = f0[opp l] + f0[opp l].  Per-cell sums in T, cell total in float64.
    """
    f0c = store.decode(f0, T)
    edge = (bc_mask[0] == bc_id) & (~missing[0])
    miss = missing[:, edge]
    fc = f0c[:, edge]
    force = []
    for d in range(lat.d):
        m = np.zeros(fc.shape[1], dtype=T)
        for l in range(lat.q):
            o = lat.opp[l]
            phi = fc[o] + fc[o]
            if lat.c[d, o] == 1:
                m = np.where(miss[l], m + phi, m)
            elif lat.c[d, o] == -1:
                m = np.where(miss[l], m - phi, m)
        force.append(np.sum(m.astype(np.float64)))
    return np.array(force)


def total_mass(lat, store, f, bc_mask, T=np.float64):
    """Sum over non-skipped cells of sum_l f_l (per cell in T, total in float64)."""
    fc = store.decode(f, T)
    acc = fc[0].copy()
    for l in range(1, lat.q):
        acc = acc + fc[l]
    keep = bc_mask[0] != 255
    return float(np.sum(acc[keep].astype(np.float64)))
