"""Macroscopic read-out rho, u (xlb/operator/macroscopic/macroscopic.py:13-66).

``Macroscopic()(f, rho, u)`` fills rho (1, *shape) and u (d, *shape) in the
compute type from a population field, as XLB's Warp implementation (:289-296);
rho and u are allocated when omitted.
"""

import torch

from xlb_gb300 import _lib
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc, spatial_shape


class Macroscopic(Operator):
    def cuda_implementation(self, f, rho=None, u=None):
        q, d = self.velocity_set.q, self.velocity_set.d
        if f.shape[0] != q or f.dtype != self.store_dtype or not f.is_contiguous() or f.device.type != "cuda":
            raise ValueError("f must be a contiguous CUDA tensor (q, ...) in the store dtype")
        cdt = self.compute_dtype
        if rho is None:
            rho = torch.empty((1,) + tuple(f.shape[1:]), dtype=cdt, device=f.device)
        if u is None:
            u = torch.empty((d,) + tuple(f.shape[1:]), dtype=cdt, device=f.device)
        for name, t, card in (("rho", rho, 1), ("u", u, d)):
            if t.dtype != cdt or t.shape[0] != card or t.numel() != card * f[0].numel() or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous ({card}, ...) tensor of dtype {cdt}")
        desc = make_desc(self.velocity_set, self.precision_policy, spatial_shape(self.velocity_set, f.shape[1:]))
        _lib.check(_lib.load().xlbg_macroscopic(desc, _lib.ptr(f), _lib.ptr(rho), _lib.ptr(u), _lib.stream_handle()))
        return rho, u
