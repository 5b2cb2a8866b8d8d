"""Global defaults, as xlb/default_config.py:7-26 (``DefaultConfig`` + ``init``)."""

from dataclasses import dataclass

from xlb_gb300.compute_backend import ComputeBackend


@dataclass
class DefaultConfig:
    default_precision_policy = None
    velocity_set = None
    default_backend = None


def init(velocity_set, default_backend=ComputeBackend.CUDA, default_precision_policy=None):
    """Set the process-wide velocity set, backend and precision policy.

    Same signature as XLB's ``xlb.init``.  Any backend value maps to the CUDA
    backend; there is no other.
    """
    if default_backend not in (ComputeBackend.CUDA,):
        raise ValueError(f"Unsupported compute backend: {default_backend}")
    DefaultConfig.velocity_set = velocity_set
    DefaultConfig.default_backend = ComputeBackend.CUDA
    DefaultConfig.default_precision_policy = default_precision_policy
    if velocity_set is not None and velocity_set.precision_policy is None:
        velocity_set.precision_policy = default_precision_policy


def default_backend():
    return DefaultConfig.default_backend
