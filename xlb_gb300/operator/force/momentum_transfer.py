"""MomentumTransfer -- XLB's momentum-exchange force operator
(xlb/operator/force/momentum_transfer.py:14-176), same constructor and call:

    momentum_transfer = MomentumTransfer(no_slip_bc)
    force = momentum_transfer(f_0, f_1, bc_mask, missing_mask)   # after the step's swap
    drag, lift = force[0], force[2]                               # windtunnel_3d.py:201-203

with torch CUDA tensors in place of ``wp.array``.  The sum runs in one CUDA
kernel (``xlbg_momentum_transfer``) over the BC's edge cells with per-cell sums
in the compute type and the sum over cells in FP64; XLB accumulates FP32
atomics.  Like XLB's Warp path (:164-176) the call returns a numpy array of d
values and synchronises with the device to read it.  ``f_1`` is accepted for
API compatibility and not read (XLB does not read it either for the no-slip
BCs).  For a force every step without a separate pass, use the stepper's
``step_with_diagnostics``, which fuses the same sum into the step.
"""

import numpy as np
import torch

from xlb_gb300 import _lib
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc, spatial_shape

_NO_SLIP = ("HalfwayBounceBackBC", "FullwayBounceBackBC")


class MomentumTransfer(Operator):
    def __init__(self, no_slip_bc_instance, velocity_set=None, precision_policy=None, compute_backend=None):
        if type(no_slip_bc_instance).__name__ not in _NO_SLIP:
            raise ValueError(
                f"MomentumTransfer needs a no-slip bounce-back BC ({', '.join(_NO_SLIP)}), "
                f"got {type(no_slip_bc_instance).__name__}"
            )
        self.no_slip_bc_instance = no_slip_bc_instance
        super().__init__(velocity_set, precision_policy, compute_backend)
        self._slots = None

    def cuda_implementation(self, f_0, f_1, bc_mask, missing_mask, out=None):
        """Force on the BC from the post-collision state f_0 (a numpy array of
        d float64 values).  With ``out`` (a float64 CUDA tensor of 4 values) the
        result [0, F_x, F_y, F_z] is written there and the call returns without
        synchronising."""
        vs = self.velocity_set
        shape = tuple(f_0.shape[1:])
        for name, t, card, dt in (
            ("f_0", f_0, vs.q, self.store_dtype),
            ("bc_mask", bc_mask, 1, torch.uint8),
            ("missing_mask", missing_mask, vs.q, torch.bool),
        ):
            if not isinstance(t, torch.Tensor) or t.device.type != "cuda" or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous CUDA tensor")
            if t.dtype != dt or t.shape[0] != card or tuple(t.shape[1:]) != shape:
                raise ValueError(f"{name} must be ({card}, {', '.join(map(str, shape))}) of dtype {dt}")
        dev = f_0.device
        if self._slots is None or self._slots.device != dev:
            self._slots = torch.zeros(_lib.DIAG_SLOTS * 4, dtype=torch.float64, device=dev)
        res = out if out is not None else torch.empty(4, dtype=torch.float64, device=dev)
        desc = make_desc(vs, self.precision_policy, spatial_shape(vs, shape))
        with torch.cuda.device(dev):
            _lib.check(
                _lib.load().xlbg_momentum_transfer(
                    desc, _lib.ptr(f_0), _lib.ptr(bc_mask), _lib.ptr(missing_mask.view(torch.uint8)),
                    int(self.no_slip_bc_instance.id), _lib.ptr(self._slots), _lib.ptr(res), _lib.stream_handle(),
                )
            )
        if out is not None:
            return out
        return res[1 : 1 + vs.d].cpu().numpy()
