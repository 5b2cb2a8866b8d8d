"""IncompressibleNavierStokesStepper -- the drop-in for XLB's fused stepper.

Same constructor, ``prepare_fields`` and call signature as
xlb/operator/stepper/nse_stepper.py:25-98 and :385-392:

    stepper = IncompressibleNavierStokesStepper(grid, boundary_conditions, collision_type="BGK")
    f_0, f_1, bc_mask, missing_mask = stepper.prepare_fields()
    for i in range(n):
        f_0, f_1 = stepper(f_0, f_1, bc_mask, missing_mask, omega, i)
        f_0, f_1 = f_1, f_0

with torch CUDA tensors in place of ``wp.array``.  Each call launches the fused
sm_103a kernel through ``xlbg_step`` on torch's current stream and returns
without synchronising.  Like XLB, a call writes f_1 and, at ZouHe / Regularized
cells, writes the BC aux values back into f_0.

``missing_mask`` keeps XLB's bool (q, nx, ny, nz) form.  The kernel reads a
packed uint32 per cell instead; the packing happens once and is cached against
the mask tensor (the tensor object and its version counter), so modifying the
mask in place -- by torch ops or by the maskers -- triggers a repack.
"""

import weakref

import numpy as np
import torch

from xlb_gb300 import _lib
from xlb_gb300.default_config import DefaultConfig
from xlb_gb300.helper.check_boundary_overlaps import check_bc_overlaps
from xlb_gb300.operator.boundary_masker import IndicesBoundaryMasker, MeshBoundaryMasker
from xlb_gb300.operator.operator import Operator
from xlb_gb300.operator.stepper.desc import make_desc
from xlb_gb300.precision_policy import Precision


class Stepper(Operator):
    """Base stepper (xlb/operator/stepper/stepper.py:6-34)."""

    def __init__(self, grid, boundary_conditions):
        self.grid = grid
        self.boundary_conditions = list(boundary_conditions)
        super().__init__(DefaultConfig.velocity_set, DefaultConfig.default_precision_policy, DefaultConfig.default_backend)

    def prepare_fields(self, initializer=None):
        raise NotImplementedError("Subclasses must implement prepare_fields()")


class IncompressibleNavierStokesStepper(Stepper):
    def __init__(
        self,
        grid,
        boundary_conditions=[],
        collision_type="BGK",
        streaming_scheme="pull",
        forcing_scheme="exact_difference",
        force_vector=None,
    ):
        super().__init__(grid, boundary_conditions)
        if collision_type == "BGK":
            # The shifted FP16/BF16 forms have no XLB counterpart and run BGK on the
            # stored deviations (same equations, pair form; their SR variants round
            # the stores stochastically); the others keep XLB's order.
            pp = self.precision_policy
            self.collision_code = (_lib.BGK_SHIFTED_SR if pp.stochastic else _lib.BGK_SHIFTED) if pp.shifted else _lib.BGK
        elif collision_type == "BGK_SHIFTED":
            pp = self.precision_policy
            if not (pp.shifted or (pp.store_code, pp.compute_code) == (0, 0)):
                raise ValueError("BGK_SHIFTED needs FP32 compute with a shifted or FP32 store "
                                 "(FP32FP16S, FP32BF16S, FP32FP32)")
            self.collision_code = _lib.BGK_SHIFTED_SR if pp.stochastic else _lib.BGK_SHIFTED
        elif collision_type == "BGK_PAIR":
            if self.precision_policy.stochastic:
                raise ValueError("stochastic rounding is defined for BGK on the stored deviations only")
            self.collision_code = _lib.BGK_PAIR
        elif collision_type == "KBC":
            if self.precision_policy.stochastic:
                raise ValueError("stochastic rounding is defined for BGK on the stored deviations only")
            if (self.velocity_set.d, self.velocity_set.q) == (3, 19):
                raise NotImplementedError(f"Velocity set not supported for KBC: {self.velocity_set}")
            self.collision_code = _lib.KBC
        else:
            raise NotImplementedError(f"collision_type {collision_type!r} is not on this path (BGK, BGK_PAIR, BGK_SHIFTED, KBC)")
        if force_vector is not None:
            raise NotImplementedError("forced collision is not on this path")
        if streaming_scheme != "pull":
            raise ValueError(f"Unknown or unimplemented streaming scheme: {streaming_scheme}")
        self.collision_type = collision_type
        self.streaming_scheme = streaming_scheme
        if grid.dim != self.velocity_set.d:
            raise ValueError(f"{grid.dim}D grid with the {self.velocity_set} velocity set")
        shape3 = tuple(grid.shape) if grid.dim == 3 else tuple(grid.shape) + (1,)
        self.desc = make_desc(self.velocity_set, self.precision_policy, shape3, self.collision_code, self.boundary_conditions)
        self._lib = _lib.load()
        self._rec_ids = [bc.id for bc in self.boundary_conditions if bc.needs_aux_recovery]
        self._cache_key = None
        self._cache = None
        self._diag_slots = None
        # ids of (f_0, f_1, bc_mask, missing_mask) -> (weak reference, data pointer, shape, strides) of each,
        # for argument tuples that passed _check
        self._checked = {}

    # ------------------------------------------------------------------ set-up

    def prepare_fields(self, initializer=None):
        """Allocate and initialise (f_0, f_1, bc_mask, missing_mask) (nse_stepper.py:58-98)."""
        from xlb_gb300.helper.nse_solver import create_nse_fields
        from xlb_gb300.helper.initializers import initialize_eq

        _, f_0, f_1, missing_mask, bc_mask = create_nse_fields(
            grid=self.grid, velocity_set=self.velocity_set, precision_policy=self.precision_policy
        )
        if initializer is not None:
            f_0 = initializer(self.grid, self.velocity_set, self.precision_policy, self.compute_backend)
        else:
            f_0 = initialize_eq(f_0, self.grid, self.velocity_set, self.precision_policy, self.compute_backend)
        f_1.copy_(f_0)
        bc_mask, missing_mask = self._process_boundary_conditions(self.boundary_conditions, bc_mask, missing_mask)
        f_0, f_1 = self._initialize_auxiliary_data(self.boundary_conditions, f_0, f_1, bc_mask, missing_mask)
        return f_0, f_1, bc_mask, missing_mask

    def _process_boundary_conditions(self, boundary_conditions, bc_mask, missing_mask):
        check_bc_overlaps(boundary_conditions, self.velocity_set.d)
        with_vertices = [bc for bc in boundary_conditions if bc.mesh_vertices is not None]
        with_indices = [bc for bc in boundary_conditions if bc.indices is not None]
        if with_indices:
            masker = IndicesBoundaryMasker(self.velocity_set, self.precision_policy)
            bc_mask, missing_mask = masker(with_indices, bc_mask, missing_mask)
        if self.velocity_set.d == 3 and with_vertices:
            mesh_masker = MeshBoundaryMasker(self.velocity_set, self.precision_policy)
            for bc in with_vertices:
                bc_mask, missing_mask = mesh_masker(bc, bc_mask, missing_mask)
        return bc_mask, missing_mask

    def _initialize_auxiliary_data(self, boundary_conditions, f_0, f_1, bc_mask, missing_mask):
        """Prescribed values into f_1[0] at each ZouHe / Regularized cell
        (boundary_condition.py:130-159, nse_stepper.py:129-135).  Stored raw in
        the store type, also for the shifted forms."""
        cdt = self.precision_policy.compute_precision.torch_dtype
        for bc in boundary_conditions:
            if not (bc.needs_aux_init and not bc.is_initialized_with_aux_data):
                continue
            lin = torch.nonzero(bc_mask.view(-1) == bc.id).view(-1)
            if lin.numel() == 0:
                bc.is_initialized_with_aux_data = True
                continue
            idx3 = np.array(np.unravel_index(lin.cpu().numpy(), tuple(bc_mask.shape[1:])))
            vals = torch.as_tensor(bc.aux_values(idx3), dtype=torch.float64, device=f_1.device)
            f_1[0].view(-1)[lin] = vals.to(cdt).to(f_1.dtype)
            bc.is_initialized_with_aux_data = True
        return f_0, f_1

    # ------------------------------------------------------------------ checks

    def _check(self, f_0, f_1, bc_mask, missing_mask):
        """Type, device, shape, dtype and layout of the four fields.  A tensor
        that passed once is not checked again while it is the same object with
        the same storage pointer, shape and strides in the same argument position
        (dtype and device cannot change in place), so the caller's swap loop
        (two argument tuples) pays one lookup a step."""
        args = (f_0, f_1, bc_mask, missing_mask)
        key = (id(f_0), id(f_1), id(bc_mask), id(missing_mask))
        e = self._checked.get(key)
        if e is not None and all(r() is t and t.data_ptr() == p and t.shape == sh and t.stride() == sd
                                 for t, (r, p, sh, sd) in zip(args, e)):
            return
        self._check_full(f_0, f_1, bc_mask, missing_mask)
        if len(self._checked) > 16:
            self._checked.clear()
        self._checked[key] = tuple((weakref.ref(t), t.data_ptr(), t.shape, t.stride()) for t in args)

    def _check_full(self, f_0, f_1, bc_mask, missing_mask):
        q = self.velocity_set.q
        fshape = (q,) + tuple(self.grid.field_shape)
        sdt = self.precision_policy.store_precision.torch_dtype
        for name, t, shape, dt in (
            ("f_0", f_0, fshape, sdt),
            ("f_1", f_1, fshape, sdt),
            ("bc_mask", bc_mask, (1,) + fshape[1:], torch.uint8),
            ("missing_mask", missing_mask, fshape, torch.bool),
        ):
            if not isinstance(t, torch.Tensor):
                raise TypeError(f"{name} must be a torch tensor")
            if t.device.type != "cuda":
                raise ValueError(f"{name} must be on a CUDA device")
            if tuple(t.shape) != shape:
                raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {shape}")
            if t.dtype != dt:
                raise TypeError(f"{name} has dtype {t.dtype}, expected {dt}")
            if not t.is_contiguous():
                raise ValueError(f"{name} must be contiguous")

    def _aux_state(self, bc_mask, missing_mask):
        """(miss_bits, rec_cells, rec_scratch), cached against the two masks.

        The cache holds weak references to the two mask tensors and their
        version counters: another tensor object (even one reusing a freed
        mask's memory) or an in-place change (torch ops bump the counter; the
        maskers bump it after their C-ABI writes) triggers a repack."""
        key = self._cache_key
        if (
            key is not None
            and key[0]() is missing_mask
            and key[1] == missing_mask._version
            and key[2]() is bc_mask
            and key[3] == bc_mask._version
        ):
            return self._cache
        n = self.grid.num_cells
        bits = torch.empty(n, dtype=torch.int32, device=bc_mask.device)
        _lib.check(self._lib.xlbg_pack_missing(self.desc, _lib.ptr(missing_mask), _lib.ptr(bits), _lib.stream_handle()))
        rec_cells, scratch = None, None
        if self._rec_ids:
            ids = torch.tensor(self._rec_ids, dtype=torch.uint8, device=bc_mask.device)
            rec_cells = torch.nonzero(torch.isin(bc_mask.view(-1), ids)).view(-1).to(torch.int64).contiguous()
            scratch = torch.empty(max(1, rec_cells.numel()) * self.velocity_set.q, dtype=self.store_dtype, device=bc_mask.device)
        self._cache_key = (weakref.ref(missing_mask), missing_mask._version, weakref.ref(bc_mask), bc_mask._version)
        self._cache = (bits, rec_cells, scratch)
        return self._cache

    def _rec_args(self, rec_cells, scratch):
        if rec_cells is None or rec_cells.numel() == 0:
            return None, 0, None
        return _lib.ptr(rec_cells), rec_cells.numel(), _lib.ptr(scratch)

    # ------------------------------------------------------------------ stepping

    def cuda_implementation(self, f_0, f_1, bc_mask, missing_mask, omega, timestep):
        """One fused step: reads f_0, writes f_1 (and aux recovery into f_0)."""
        self._check(f_0, f_1, bc_mask, missing_mask)
        bits, rec_cells, scratch = self._aux_state(bc_mask, missing_mask)
        rc, nrec, scr = self._rec_args(rec_cells, scratch)
        rc_ = self._lib.xlbg_step(
            self.desc, f_0.data_ptr(), f_1.data_ptr(), bc_mask.data_ptr(), bits.data_ptr(), rc, nrec, scr,
            float(omega), int(timestep), _lib.raw_stream(f_0.get_device()),
        )
        if rc_:
            _lib.check(rc_)
        return f_0, f_1

    __call__ = cuda_implementation

    def run(self, f_0, f_1, bc_mask, missing_mask, omega, num_steps, timestep0=0):
        """``num_steps`` steps of the swap loop above in one C call.  Returns
        (f_0, f_1) with f_0 holding the newest state, i.e. the pair the user loop
        holds after its final swap."""
        self._check(f_0, f_1, bc_mask, missing_mask)
        bits, rec_cells, scratch = self._aux_state(bc_mask, missing_mask)
        rc, nrec, scr = self._rec_args(rec_cells, scratch)
        _lib.check(
            self._lib.xlbg_run(
                self.desc, _lib.ptr(f_0), _lib.ptr(f_1), _lib.ptr(bc_mask), _lib.ptr(bits), rc, nrec, scr,
                float(omega), int(timestep0), int(num_steps), _lib.raw_stream(f_0.get_device()),
            )
        )
        return (f_1, f_0) if num_steps % 2 else (f_0, f_1)

    def step_with_diagnostics(self, f_0, f_1, bc_mask, missing_mask, omega, timestep, force_bc=None, out=None):
        """One step that also returns a float64 CUDA tensor of 4 values:
        [mass of the new state f_1, force on ``force_bc`` (x, y[, z]) evaluated
        on the input state f_0] -- the force is what XLB's MomentumTransfer
        returns for f_0 after the previous step's swap."""
        self._check(f_0, f_1, bc_mask, missing_mask)
        bits, rec_cells, scratch = self._aux_state(bc_mask, missing_mask)
        rc, nrec, scr = self._rec_args(rec_cells, scratch)
        if self._diag_slots is None or self._diag_slots.device != f_0.device:
            self._diag_slots = torch.zeros(_lib.DIAG_SLOTS * 4, dtype=torch.float64, device=f_0.device)
        if out is None:
            out = torch.empty(4, dtype=torch.float64, device=f_0.device)
        force_id = -1 if force_bc is None else int(force_bc.id)
        _lib.check(
            self._lib.xlbg_step_diag(
                self.desc, _lib.ptr(f_0), _lib.ptr(f_1), _lib.ptr(bc_mask), _lib.ptr(bits), rc, nrec, scr,
                float(omega), int(timestep), force_id, _lib.ptr(self._diag_slots), _lib.ptr(out),
                _lib.raw_stream(f_0.get_device()),
            )
        )
        return f_0, f_1, out

    def differentiable(self, bc_mask, missing_mask, omega, num_steps, checkpoint_every=100, use_graphs=True):
        """``num_steps`` steps as a differentiable map (f_init, aux_values) -> f_final,
        backed by the hand-written adjoint (see ``DifferentiableRun``)."""
        from xlb_gb300.operator.stepper.adjoint import DifferentiableRun

        return DifferentiableRun(self, bc_mask, missing_mask, omega, num_steps, checkpoint_every, use_graphs)


__all__ = ["Stepper", "IncompressibleNavierStokesStepper", "Precision"]
