"""bc_mask / missing_mask from BC index lists (set-up, not timed).

Follows XLB's Warp IndicesBoundaryMasker (indices_boundary_masker.py:103-224):
each in-domain index gets its BC id; direction l is missing where the pull
source index - c_l leaves the domain; for BCs that need padding and indices in
the domain interior (:29-40), each in-bounds direction marks the push neighbour
index + c_l as missing in l and gives it the BC id (l = 0 marks the cell
itself).  XLB runs all BCs in one racy launch; here BCs are applied in list
order on the GPU stream, so where two BCs touch the same cell the later one
wins.
"""

import numpy as np
import torch

from xlb_gb300.operator.operator import Operator


class IndicesBoundaryMasker(Operator):
    def are_indices_in_interior(self, indices, shape):
        d = self.velocity_set.d
        shape_array = np.array(shape)
        return np.all((indices[:d] > 0) & (indices[:d] < shape_array[:d, np.newaxis] - 1), axis=0)

    def cuda_implementation(self, bclist, bc_mask, missing_mask, start_index=None):
        vs = self.velocity_set
        d, q = vs.d, vs.q
        dev = bc_mask.device
        shp = np.array(bc_mask.shape[1:])
        for bc in bclist:
            if bc.indices is None:
                raise ValueError(f'Please specify indices associated with the {bc.__class__.__name__} BC using keyword "indices"!')
            idx = bc.index_array.copy()
            if start_index is not None:
                idx = idx - np.asarray(start_index)[:, None]
            if idx.shape[0] == 2:
                idx = np.vstack([idx, np.zeros(idx.shape[1], dtype=np.int64)])
            inb = np.all((idx >= 0) & (idx < shp[:, None]), axis=0)
            interior_all = self.are_indices_in_interior(idx, tuple(shp)) if bc.needs_padding else np.zeros(idx.shape[1], dtype=bool)
            idx = idx[:, inb]
            interior = interior_all[inb]
            own = torch.as_tensor(idx, device=dev)
            bc_mask[0, own[0], own[1], own[2]] = bc.id
            for l in range(q):
                c3 = np.zeros(3, dtype=np.int64)
                c3[:d] = vs.c[:, l]
                pull = idx - c3[:, None]
                pull[d:] = 0
                pin = np.all((pull >= 0) & (pull < shp[:, None]), axis=0)
                out = torch.as_tensor(np.nonzero(~pin)[0], device=dev)
                if out.numel():
                    missing_mask[l, own[0, out], own[1, out], own[2, out]] = True
                sel = pin & interior
                if sel.any():
                    push = torch.as_tensor(idx[:, sel] + c3[:, None], device=dev)
                    missing_mask[l, push[0], push[1], push[2]] = True
                    bc_mask[0, push[0], push[1], push[2]] = bc.id
        return bc_mask, missing_mask
