"""Lattice velocity sets (D2Q9, D3Q19, D3Q27).

The direction ORDER is part of the public API: populations are stored as
``f[l, ...]`` with ``l`` indexing these tables, exactly as XLB does
(xlb/velocity_set/d2q9.py:18-21, d3q19.py:19, d3q27.py:19).  The derived tables
follow xlb/velocity_set/velocity_set.py:

* ``opp_indices``  -- index of -c_l              (velocity_set.py:167-180)
* ``cc``           -- packed c_a c_b, a <= b     (velocity_set.py:140-165)
* ``qi``           -- cc - cs^2 I, off-diagonals doubled (velocity_set.py:124-138)
* ``main/right/left_indices``                    (velocity_set.py:182-221)

The CUDA kernels carry their own compile-time copies of c, w and opp; a CPU
test checks them against these tables through ``xlbg_lattice_tables``.
"""

import itertools
import math

import numpy as np


class VelocitySet:
    """Base class.  ``c`` has shape (d, q) and ``w`` shape (q,), as in XLB."""

    def __init__(self, d, q, c, w, precision_policy=None, compute_backend=None):
        self.d = d
        self.q = q
        self.precision_policy = precision_policy
        self.compute_backend = compute_backend
        self._c = np.asarray(c, dtype=np.int64)
        self._w = np.asarray(w, dtype=np.float64)
        if self._c.shape != (d, q) or self._w.shape != (q,):
            raise ValueError("velocity table has the wrong shape")
        self._opp_indices = self._build_opposite()
        self._cc = self._build_cc()
        self._qi = self._build_qi()
        self._c_float = self._c.astype(np.float64)
        self.cs = np.float64(math.sqrt(3) / 3.0)
        self.cs2 = np.float64(1.0 / 3.0)
        self.inv_cs2 = np.float64(3.0)
        cols = self._c.T
        l1 = np.abs(cols).sum(axis=1)
        self.main_indices = np.nonzero(l1 == 1)[0]
        self.right_indices = np.nonzero(cols[:, 0] == 1)[0]
        self.left_indices = np.nonzero(cols[:, 0] == -1)[0]

    # numpy views (XLB exposes backend arrays under the same names)
    @property
    def c(self):
        return self._c

    @property
    def w(self):
        return self._w

    @property
    def opp_indices(self):
        return self._opp_indices

    @property
    def cc(self):
        return self._cc

    @property
    def qi(self):
        return self._qi

    @property
    def c_float(self):
        return self._c_float

    def _build_opposite(self):
        cols = [tuple(v) for v in self._c.T.tolist()]
        lookup = {v: i for i, v in enumerate(cols)}
        return np.array([lookup[tuple(-x for x in v)] for v in cols], dtype=np.int64)

    def _build_cc(self):
        nt = self.d * (self.d + 1) // 2
        cc = np.zeros((self.q, nt))
        k = 0
        for a in range(self.d):
            for b in range(a, self.d):
                cc[:, k] = self._c[a] * self._c[b]
                k += 1
        return cc

    def _build_qi(self):
        if self.d == 3:
            diag, offdiag = (0, 3, 5), (1, 2, 4)
        elif self.d == 2:
            diag, offdiag = (0, 2), (1,)
        else:
            raise ValueError(f"dim = {self.d} not supported")
        qi = self._cc.copy()
        qi[:, diag] += -1.0 / 3.0
        qi[:, offdiag] *= 2.0
        return qi

    def __repr__(self):
        return f"D{self.d}Q{self.q}"

    __str__ = __repr__

    def __eq__(self, other):
        return isinstance(other, VelocitySet) and other.d == self.d and other.q == self.q

    def __hash__(self):
        return hash((self.d, self.q))


class D2Q9(VelocitySet):
    """2D, nine velocities (xlb/velocity_set/d2q9.py:18-24)."""

    def __init__(self, precision_policy=None, compute_backend=None):
        cx = [0, 0, 0, 1, -1, 1, -1, 1, -1]
        cy = [0, 1, -1, 0, 1, -1, 0, 1, -1]
        w = [4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 9, 1 / 36, 1 / 36]
        super().__init__(2, 9, np.array([cx, cy]), w, precision_policy, compute_backend)


def _weights_by_norm(c, table):
    return np.array([table[int(np.abs(c[:, i]).sum())] for i in range(c.shape[1])])


class D3Q19(VelocitySet):
    """3D, nineteen velocities: product([0,-1,1]) with |c|_1 <= 2 (d3q19.py:19-28)."""

    def __init__(self, precision_policy=None, compute_backend=None):
        c = np.array([v for v in itertools.product([0, -1, 1], repeat=3) if sum(map(abs, v)) <= 2]).T
        w = _weights_by_norm(c, {0: 1.0 / 3.0, 1: 1.0 / 18.0, 2: 1.0 / 36.0})
        super().__init__(3, 19, c, w, precision_policy, compute_backend)


class D3Q27(VelocitySet):
    """3D, twenty-seven velocities: product([0,-1,1], repeat=3) (d3q27.py:19-30)."""

    def __init__(self, precision_policy=None, compute_backend=None):
        c = np.array(list(itertools.product([0, -1, 1], repeat=3))).T
        w = _weights_by_norm(c, {0: 8.0 / 27.0, 1: 2.0 / 27.0, 2: 1.0 / 54.0, 3: 1.0 / 216.0})
        super().__init__(3, 27, c, w, precision_policy, compute_backend)


LATTICE_CODE = {(2, 9): 0, (3, 19): 1, (3, 27): 2}


def lattice_code(velocity_set):
    """Integer lattice id used by the C-ABI (``xlbg_lattice`` in include/xlbg.h)."""
    return LATTICE_CODE[(velocity_set.d, velocity_set.q)]
