"""Grid objects: shape, face indices and field allocation.

Mirrors xlb/grid/grid.py:9-86 and xlb/grid/warp_grid.py:17-32.  Fields are
torch CUDA tensors in XLB's Warp layout: (cardinality, nx, ny, nz), with a
trailing singleton axis for 2D grids.
"""

from typing import Tuple

import numpy as np
import torch

from xlb_gb300.default_config import DefaultConfig


def grid_factory(shape: Tuple[int, ...], compute_backend=None, device=None):
    """Return a grid for ``shape`` (2 or 3 entries), as xlb.grid.grid_factory."""
    return Grid(tuple(int(s) for s in shape), device=device)


class Grid:
    def __init__(self, shape, device=None):
        if len(shape) not in (2, 3):
            raise ValueError("grid shape must have 2 or 3 entries")
        if any(s <= 0 for s in shape):
            raise ValueError("grid shape must be positive")
        self.shape = shape
        self.dim = len(shape)
        self.device = torch.device(device) if device is not None else torch.device("cuda")

    @property
    def field_shape(self):
        """Spatial part of a field's shape: (nx, ny, nz) or (nx, ny, 1)."""
        return self.shape if self.dim == 3 else self.shape + (1,)

    @property
    def num_cells(self):
        return int(np.prod(self.shape))

    def bounding_box_indices(self, remove_edges=False):
        """Face indices, as grid.py:34-86: keys bottom/top/left/right (+front/back
        in 3D); each value is a list of d index lists.  In 3D "top" is z = nz-1 and
        "left" is x = 0; in 2D "top" is y = ny-1."""
        origin = np.array([0, 0, 0])
        bounds = np.array(self.shape)
        if remove_edges:
            origin += 1
            bounds -= 1
        sx = slice(origin[0], bounds[0])
        sy = slice(origin[1], bounds[1])
        grid = np.indices(self.shape)
        if self.dim == 2:
            nx, ny = self.shape
            faces = {
                "bottom": grid[:, sx, 0],
                "top": grid[:, sx, ny - 1],
                "left": grid[:, 0, sy],
                "right": grid[:, nx - 1, sy],
            }
        else:
            nx, ny, nz = self.shape
            sz = slice(origin[2], bounds[2])
            faces = {
                "bottom": grid[:, sx, sy, 0].reshape(3, -1),
                "top": grid[:, sx, sy, nz - 1].reshape(3, -1),
                "left": grid[:, 0, sy, sz].reshape(3, -1),
                "right": grid[:, nx - 1, sy, sz].reshape(3, -1),
                "front": grid[:, sx, 0, sz].reshape(3, -1),
                "back": grid[:, sx, ny - 1, sz].reshape(3, -1),
            }
        return {k: v.tolist() for k, v in faces.items()}

    def create_field(self, cardinality, dtype=None, fill_value=None):
        """Zero- or value-filled field (cardinality, *field_shape)."""
        if dtype is None:
            dtype = DefaultConfig.default_precision_policy.store_precision
        tdtype = dtype.torch_dtype if hasattr(dtype, "torch_dtype") else dtype
        shape = (int(cardinality),) + self.field_shape
        if fill_value is None:
            return torch.zeros(shape, dtype=tdtype, device=self.device)
        return torch.full(shape, fill_value, dtype=tdtype, device=self.device)


# XLB exposes the backend-specific class name; both names refer to the CUDA grid.
WarpGrid = Grid
CudaGrid = Grid
