"""Field allocation for the stepper (xlb/helper/nse_solver.py:7-41)."""

from xlb_gb300.default_config import DefaultConfig
from xlb_gb300.grid import grid_factory
from xlb_gb300.precision_policy import Precision


def create_nse_fields(grid_shape=None, grid=None, velocity_set=None, compute_backend=None, precision_policy=None):
    """Returns (grid, f_0, f_1, missing_mask, bc_mask) as CUDA tensors."""
    velocity_set = velocity_set or DefaultConfig.velocity_set
    precision_policy = precision_policy or DefaultConfig.default_precision_policy
    if grid is None:
        if grid_shape is None:
            raise ValueError("grid_shape must be provided when grid is None")
        grid = grid_factory(grid_shape)
    f_0 = grid.create_field(cardinality=velocity_set.q, dtype=precision_policy.store_precision)
    f_1 = grid.create_field(cardinality=velocity_set.q, dtype=precision_policy.store_precision)
    missing_mask = grid.create_field(cardinality=velocity_set.q, dtype=Precision.BOOL)
    bc_mask = grid.create_field(cardinality=1, dtype=Precision.UINT8)
    return grid, f_0, f_1, missing_mask, bc_mask
