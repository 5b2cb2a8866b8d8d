"""Duplicate-index check before masking (xlb/helper/check_boundary_overlaps.py:5-24).

XLB's Warp path raises on duplicates inside one BC and across BCs; so does this.
"""

import numpy as np


def check_bc_overlaps(bclist, dim, compute_backend=None):
    index_list = [[] for _ in range(dim)]
    for bc in bclist:
        if bc.indices is None:
            continue
        idx = bc.index_array[:dim]
        if np.unique(idx, axis=-1).shape[-1] != idx.shape[-1]:
            raise ValueError(f"Boundary condition {bc.__class__.__name__} has duplicate indices!")
        for d in range(dim):
            index_list[d] += idx[d].tolist()
    if index_list[0]:
        arr = np.array(index_list)
        if np.unique(arr, axis=-1).shape[-1] != arr.shape[-1]:
            raise ValueError("Boundary condition list containes duplicate indices!")
