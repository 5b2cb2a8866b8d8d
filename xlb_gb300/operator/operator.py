"""Operator base class (xlb/operator/operator.py:10-134).

XLB resolves a backend implementation per call by signature binding
(operator.py:54-74).  Here there is one backend, so ``__call__`` goes straight
to ``cuda_implementation``; errors propagate with their own type instead of
being re-wrapped in a generic ``Exception``.
"""

from xlb_gb300.compute_backend import ComputeBackend
from xlb_gb300.default_config import DefaultConfig


class Operator:
    def __init__(self, velocity_set=None, precision_policy=None, compute_backend=None):
        self.velocity_set = velocity_set or DefaultConfig.velocity_set
        self.precision_policy = precision_policy or DefaultConfig.default_precision_policy
        self.compute_backend = ComputeBackend.CUDA
        if compute_backend is not None and compute_backend not in ComputeBackend:
            raise ValueError(f"Compute_backend {compute_backend} is not supported")

    def __call__(self, *args, **kwargs):
        return self.cuda_implementation(*args, **kwargs)

    def cuda_implementation(self, *args, **kwargs):
        raise NotImplementedError(f"{self.__class__.__name__} has no CUDA implementation")

    # XLB's name for the same entry
    def warp_implementation(self, *args, **kwargs):
        return self.cuda_implementation(*args, **kwargs)

    @property
    def compute_dtype(self):
        return self.precision_policy.compute_precision.torch_dtype

    @property
    def store_dtype(self):
        return self.precision_policy.store_precision.torch_dtype

    @property
    def backend(self):
        import torch

        return torch

    def __repr__(self):
        return f"{self.__class__.__name__}()"
