"""ctypes wrapper of the C restatement (oracle/lbm_ref.c) -- TEST INFRASTRUCTURE ONLY.

Same semantics as lbm_oracle.step for the FP32FP32 and FP64FP64 policies, with
OpenMP across cells.  Used by tests at sizes the numpy oracle is too slow for
and by bench.py as the CPU baseline.
"""

import ctypes

import numpy as np

from oracle import build_oracle

_lib = None
KINDS = {
    "fullway_bb": 1, "halfway_bb": 2, "equilibrium": 3, "zouhe_velocity": 4, "zouhe_pressure": 5,
    "regularized_velocity": 6, "regularized_pressure": 7, "extrapolation": 8,
}
LATTICE = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}


def load():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        lib = ctypes.CDLL(path)
        P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        for sfx in ("f32", "f64"):
            fn = getattr(lib, f"lbm_ref_step_{sfx}")
            fn.argtypes = [I, I, I64, I64, I64, P, P, P, P, I, P, P, P, P, D, I]
            fn.restype = I
        lib.lbm_ref_max_threads.restype = I
        _lib = lib
    return _lib


def max_threads():
    return load().lbm_ref_max_threads()


class Stepper:
    """Holds the BC tables and the packed missing bits for repeated steps."""

    def __init__(self, lat, shape, bc_mask, missing, bcs, collision="BGK", T=np.float32, threads=0):
        self.lat, self.T, self.threads = lat, T, threads
        self.s3 = tuple(shape) if len(shape) == 3 else tuple(shape) + (1,)
        self.collision = {"BGK": 0, "KBC": 1, "BGK_PAIR": 2}[collision]
        self.bc_mask = np.ascontiguousarray(bc_mask, dtype=np.uint8)
        bits = np.zeros(self.s3, dtype=np.uint32)
        for l in range(lat.q):
            bits |= missing[l].astype(np.uint32) << np.uint32(l)
        self.bits = bits
        self.ids = np.array([b.id for b in bcs] or [0], dtype=np.int32)
        self.kinds = np.array([KINDS[b.kind] for b in bcs] or [0], dtype=np.int32)
        self.rhos = np.array([b.rho for b in bcs] or [0.0], dtype=np.float64)
        self.us = np.array([list(b.u) + [0.0] * (3 - len(b.u)) for b in bcs] or [[0.0] * 3], dtype=np.float64).reshape(-1)
        self.nbc = len(bcs)

    def step(self, f0, f1, omega):
        """In place: f1 <- step(f0); f0 receives the aux recovery writes."""
        assert f0.dtype == self.T and f1.dtype == self.T and f0.flags.c_contiguous and f1.flags.c_contiguous
        fn = getattr(load(), "lbm_ref_step_f32" if self.T == np.float32 else "lbm_ref_step_f64")
        c = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        nx, ny, nz = self.s3
        fn(LATTICE[self.lat.name], self.collision, nx, ny, nz, c(f0), c(f1), c(self.bc_mask),
           c(self.bits), self.nbc, c(self.ids), c(self.kinds), c(self.rhos), c(self.us), float(omega), int(self.threads))

    def run(self, f0, f1, omega, steps):
        """``steps`` steps with the caller-side swap; returns (newest, other)."""
        for _ in range(steps):
            self.step(f0, f1, omega)
            f0, f1 = f1, f0
        return f0, f1


__all__ = ["Stepper", "load", "max_threads"]
