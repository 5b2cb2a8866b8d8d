"""Quadratic equilibrium operator (xlb/operator/equilibrium/quadratic_equilibrium.py:12-116).

``QuadraticEquilibrium()(rho, u, f)`` fills f with feq(rho, u) in the store
form, as XLB's Warp implementation (:382-394).  rho (1, *shape) and u
(d, *shape) are compute-type CUDA tensors; either may be None for rho = 1 /
u = 0 everywhere (the default of ``initialize_eq``).
"""


from xlb_gb300 import _lib
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc, spatial_shape


class Equilibrium(Operator):
    pass


class QuadraticEquilibrium(Equilibrium):
    def cuda_implementation(self, rho, u, f, rho0=1.0, u0=None):
        q, d = self.velocity_set.q, self.velocity_set.d
        if f.shape[0] != q or f.dtype != self.store_dtype or not f.is_contiguous() or f.device.type != "cuda":
            raise ValueError("f must be a contiguous CUDA tensor (q, ...) in the store dtype")
        desc = make_desc(self.velocity_set, self.precision_policy, spatial_shape(self.velocity_set, f.shape[1:]))
        cdt = self.compute_dtype
        for name, t, card in (("rho", rho, 1), ("u", u, d)):
            if t is not None and (t.dtype != cdt or t.shape[0] != card or t.numel() != card * f[0].numel() or not t.is_contiguous()):
                raise ValueError(f"{name} must be a contiguous ({card}, ...) tensor of dtype {cdt}")
        u0v = (_lib._D * 3)(*((list(u0) if u0 is not None else []) + [0.0] * 3)[:3])
        _lib.check(
            _lib.load().xlbg_equilibrium(desc, _lib.ptr(rho), _lib.ptr(u), float(rho0), u0v, _lib.ptr(f), _lib.stream_handle())
        )
        return f


__all__ = ["Equilibrium", "QuadraticEquilibrium"]
