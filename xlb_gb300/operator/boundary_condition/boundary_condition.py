"""Boundary-condition base class and id registry.

Mirrors xlb/operator/boundary_condition/boundary_condition.py:23-175 and
boundary_condition_registry.py:6-30.  A BC holds its id (a uint8 written into
bc_mask; 0 is fluid, 255 marks cells the stepper skips), the indices it applies
to, the step it acts in, and the flags the masker and the stepper read.  The
per-cell arithmetic itself is compiled into the fused CUDA step kernel; each
class only names its kind (``kind`` is an ``XLBG_BC_*`` code from
include/xlbg.h).
"""

from enum import Enum, auto

import numpy as np

from xlb_gb300.default_config import DefaultConfig
from xlb_gb300.operator.operator import Operator


class ImplementationStep(Enum):
    COLLISION = auto()
    STREAMING = auto()


class BoundaryConditionRegistry:
    """Global, never-reused BC ids starting at 1 (boundary_condition_registry.py:6-30)."""

    def __init__(self):
        self.id_to_bc = {}
        self.bc_to_id = {}
        self.next_id = 1

    def register_boundary_condition(self, boundary_condition):
        _id = self.next_id
        if _id > 254:
            raise RuntimeError("more than 254 boundary conditions registered; ids are uint8 and 255 is reserved")
        self.next_id += 1
        self.id_to_bc[_id] = boundary_condition
        self.bc_to_id[boundary_condition] = _id
        return _id


boundary_condition_registry = BoundaryConditionRegistry()


def _normalize_indices(indices):
    if indices is None:
        return None
    arr = np.asarray([np.asarray(v).reshape(-1) for v in indices], dtype=np.int64)
    if arr.ndim != 2 or arr.shape[0] not in (2, 3):
        raise ValueError("indices must be a list of 2 or 3 index sequences")
    return arr


class BoundaryCondition(Operator):
    kind = 0
    mesh_vertices = None  # what an instance reads after the mesh masker dropped its vertices

    def __init__(
        self,
        implementation_step,
        velocity_set=None,
        precision_policy=None,
        compute_backend=None,
        indices=None,
        mesh_vertices=None,
    ):
        self.id = boundary_condition_registry.register_boundary_condition(self.__class__.__name__ + "_" + str(hash(self)))
        super().__init__(velocity_set or DefaultConfig.velocity_set, precision_policy or DefaultConfig.default_precision_policy, compute_backend)
        self.indices = indices
        self.mesh_vertices = mesh_vertices
        self.implementation_step = implementation_step
        self.needs_padding = False
        self.needs_mesh_distance = False
        self.needs_aux_init = False
        self.is_initialized_with_aux_data = False
        self.num_of_aux_data = 0
        self.needs_aux_recovery = False

    @property
    def index_array(self):
        """indices as an int64 array of shape (d, n)."""
        return _normalize_indices(self.indices)

    def c_entry(self):
        """(id, kind, rho, u) for the C-ABI BC table."""
        return (self.id, self.kind, 0.0, (0.0, 0.0, 0.0))
