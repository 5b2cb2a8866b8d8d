"""Compute / store precision pairs.

Mirrors xlb/precision_policy.py:8-89 (``Precision`` and ``PrecisionPolicy`` with
the same member names).  Two store forms are new here:

* ``FP32FP16S`` -- populations stored as FP16 *shifted deviations*
  (f_l - w_l) * 2^14, computed in FP32 (the DDF-shifting of Lehmann et al., Phys.
  Rev. E 106, 015308 (2022); the power-of-two scale keeps small deviations out of
  FP16's subnormal range).  XLB's ``FP32FP16`` stores raw FP16 and is kept as-is.
* ``FP32BF16S`` -- f_l - w_l in BF16 (no scale: BF16 has FP32's exponent range).
* ``FP32FP16SR`` / ``FP32BF16SR`` -- the same stored values, rounded
  stochastically on store (Blackwell's ``cvt.rs`` with hashed random bits of
  the cell and time step) instead of to nearest: a per-step change smaller than
  half a 16-bit ulp then survives in expectation instead of being lost in every
  cell that sits near a steady value.

With shifted storage every population slot holds the (scaled) ``f - w_l``,
except the boundary auxiliary value that ZouHe / Regularized keep in slot 0 of
the aux buffer: that one is stored raw (unshifted), because it is a prescribed
velocity or density, not a population.
"""

from enum import Enum, auto

import numpy as np
import torch


class Precision(Enum):
    FP64 = auto()
    FP32 = auto()
    FP16 = auto()
    BF16 = auto()
    UINT8 = auto()
    BOOL = auto()

    @property
    def torch_dtype(self):
        return {
            Precision.FP64: torch.float64,
            Precision.FP32: torch.float32,
            Precision.FP16: torch.float16,
            Precision.BF16: torch.bfloat16,
            Precision.UINT8: torch.uint8,
            Precision.BOOL: torch.bool,
        }[self]

    @property
    def np_dtype(self):
        return {
            Precision.FP64: np.float64,
            Precision.FP32: np.float32,
            Precision.FP16: np.float16,
            Precision.BF16: np.float32,  # numpy has no bfloat16; host copies widen
            Precision.UINT8: np.uint8,
            Precision.BOOL: np.bool_,
        }[self]

    # XLB exposes ``wp_dtype``/``jax_dtype``; the torch dtype plays that role here.
    @property
    def wp_dtype(self):
        return self.torch_dtype


# C-ABI codes (xlbg_store / xlbg_compute in include/xlbg.h)
STORE_F32, STORE_F64, STORE_F16, STORE_F16S, STORE_BF16S = 0, 1, 2, 3, 4
COMPUTE_F32, COMPUTE_F64 = 0, 1


class PrecisionPolicy(Enum):
    FP64FP64 = auto()
    FP64FP32 = auto()
    FP64FP16 = auto()
    FP32FP32 = auto()
    FP32FP16 = auto()
    FP32FP16S = auto()
    FP32BF16S = auto()
    FP32FP16SR = auto()
    FP32BF16SR = auto()

    @property
    def compute_precision(self):
        if self in (PrecisionPolicy.FP64FP64, PrecisionPolicy.FP64FP32, PrecisionPolicy.FP64FP16):
            return Precision.FP64
        return Precision.FP32

    @property
    def store_precision(self):
        return {
            PrecisionPolicy.FP64FP64: Precision.FP64,
            PrecisionPolicy.FP64FP32: Precision.FP32,
            PrecisionPolicy.FP64FP16: Precision.FP16,
            PrecisionPolicy.FP32FP32: Precision.FP32,
            PrecisionPolicy.FP32FP16: Precision.FP16,
            PrecisionPolicy.FP32FP16S: Precision.FP16,
            PrecisionPolicy.FP32BF16S: Precision.BF16,
            PrecisionPolicy.FP32FP16SR: Precision.FP16,
            PrecisionPolicy.FP32BF16SR: Precision.BF16,
        }[self]

    @property
    def shifted(self):
        """True when populations are stored as f - w_l."""
        return self in (PrecisionPolicy.FP32FP16S, PrecisionPolicy.FP32BF16S, PrecisionPolicy.FP32FP16SR,
                        PrecisionPolicy.FP32BF16SR)

    @property
    def stochastic(self):
        """True when stores round stochastically (the shifted forms' SR variants)."""
        return self in (PrecisionPolicy.FP32FP16SR, PrecisionPolicy.FP32BF16SR)

    @property
    def store_code(self):
        if self in (PrecisionPolicy.FP32FP16S, PrecisionPolicy.FP32FP16SR):
            return STORE_F16S
        if self in (PrecisionPolicy.FP32BF16S, PrecisionPolicy.FP32BF16SR):
            return STORE_BF16S
        return {Precision.FP32: STORE_F32, Precision.FP64: STORE_F64, Precision.FP16: STORE_F16}[self.store_precision]

    @property
    def compute_code(self):
        return COMPUTE_F64 if self.compute_precision == Precision.FP64 else COMPUTE_F32

    @property
    def store_bytes(self):
        return torch.empty((), dtype=self.store_precision.torch_dtype).element_size()
