"""Compute backend enum.

XLB selects between ``JAX`` and ``WARP`` (xlb/compute_backend.py).  This
package has exactly one backend, hand-written sm_103a CUDA, named ``CUDA``.
``WARP`` is kept as an alias so that code written against XLB's Warp backend
runs unchanged; ``JAX`` is not offered.
"""

from enum import Enum


class ComputeBackend(Enum):
    CUDA = "cuda"
    WARP = "cuda"  # alias of CUDA (same member)
