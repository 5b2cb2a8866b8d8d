"""bc_mask / missing_mask from BC index lists (set-up, not timed).

Follows XLB's Warp IndicesBoundaryMasker (indices_boundary_masker.py:103-224):
each in-domain index gets its BC id; direction l is missing where the pull
source index - c_l leaves the domain; for BCs that need padding and indices in
the domain interior (:29-40), each in-bounds direction marks the push neighbour
index + c_l as missing in l and gives it the BC id (l = 0 marks the cell
itself).  The work is the CUDA kernel of ``xlbg_indices_mask``, launched once
per BC.  XLB runs all BCs in one racy launch; here BCs are applied in list
order on the GPU stream, so where two BCs touch the same cell the later one
wins.
"""

import numpy as np
import torch

from xlb_gb300 import _lib
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc


class IndicesBoundaryMasker(Operator):
    def are_indices_in_interior(self, indices, shape):
        d = self.velocity_set.d
        shape_array = np.array(shape)
        return np.all((indices[:d] > 0) & (indices[:d] < shape_array[:d, np.newaxis] - 1), axis=0)

    def cuda_implementation(self, bclist, bc_mask, missing_mask, start_index=None):
        vs = self.velocity_set
        if bc_mask.dtype != torch.uint8 or missing_mask.dtype not in (torch.bool, torch.uint8):
            raise TypeError("bc_mask must be uint8 and missing_mask bool or uint8")
        if not (bc_mask.is_cuda and missing_mask.is_cuda and bc_mask.is_contiguous() and missing_mask.is_contiguous()):
            raise ValueError("bc_mask and missing_mask must be contiguous CUDA tensors")
        shape = tuple(int(s) for s in bc_mask.shape[1:])
        if tuple(missing_mask.shape) != (vs.q,) + shape:
            raise ValueError("missing_mask must have shape (q, nx, ny[, nz]) of bc_mask's grid")
        shape3 = shape if len(shape) == 3 else shape + (1,)
        desc = make_desc(vs, self.precision_policy, shape3)
        dev = bc_mask.device
        lib = _lib.load()
        for bc in bclist:
            if bc.indices is None:
                raise ValueError(f'Please specify indices associated with the {bc.__class__.__name__} BC using keyword "indices"!')
            assert bc.mesh_vertices is None, f"Please use MeshBoundaryMasker operator if {bc.__class__.__name__} is imposed on a mesh (e.g. STL)!"
            idx = bc.index_array.copy()
            if start_index is not None:
                idx = idx - np.asarray(start_index)[:, None]
            if idx.shape[0] == 2:
                idx = np.vstack([idx, np.zeros(idx.shape[1], dtype=np.int64)])
            dev_idx = torch.as_tensor(np.ascontiguousarray(idx, dtype=np.int64), device=dev)
            with torch.cuda.device(dev):
                _lib.check(
                    lib.xlbg_indices_mask(
                        desc, _lib.ptr(dev_idx), int(idx.shape[1]), int(bc.id), 1 if bc.needs_padding else 0,
                        _lib.ptr(bc_mask), _lib.ptr(missing_mask.view(torch.uint8)), _lib.stream_handle(),
                    )
                )
            _lib.mark_written(bc_mask, missing_mask)
        return bc_mask, missing_mask
