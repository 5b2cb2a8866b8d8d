"""Differentiation of K fused steps: a torch.autograd.Function over the
hand-written adjoint kernel, with segment checkpointing.

XLB differentiates its stepper by running it under a Warp tape
(examples/out_of_core/subroutine/autodiff_stepper_subroutine.py:460-466) in
segments between stored states (examples/out_of_core/autodiff_lbm.py:64-124).
Here the same schedule runs on the C ABI:

* forward: the state at the start of every segment of ``checkpoint_every``
  steps is kept (``xlbg_forward_segment`` records each segment into a buffer
  of checkpoint_every + 1 states);
* backward: segments are replayed from their checkpoint in reverse order, each
  replay recording the segment's states, followed by ``xlbg_adjoint_segment``,
  which applies the transposed Jacobian of every step of the segment.  The last
  segment is still in the buffer after the forward pass and is not replayed.

Memory: ceil(K / k) checkpoints plus k + 1 recorded states plus two adjoint
fields, k = checkpoint_every; the recorded segment, the aux field and the
adjoint fields belong to the plan and are reused by every call.  Compute: one
forward pass, one replay (of all segments but the last) and one adjoint sweep.

Each segment's recording and reverse sweep is captured once as a CUDA graph
(the kernels of k steps in one launch) and replayed afterwards, which matters
for small grids where a step's kernels take a few microseconds.  A backward
whose recorded last segment was overwritten by a later forward replays that
segment from its checkpoint, so interleaved calls stay exact.

The state of the map is the population field; the ZouHe / Regularized
prescribed values are a separate differentiable input (one value per such
cell, in the order of ``aux_cells``), so a learnable inlet profile gets its
gradient through them.
"""

import math

import torch

from xlb_gb300 import _lib

_AUX = (_lib.BC_ZOUHE_VELOCITY, _lib.BC_ZOUHE_PRESSURE, _lib.BC_REGULARIZED_VELOCITY, _lib.BC_REGULARIZED_PRESSURE)


def _cells_of(bc_mask, ids):
    if not ids:
        return torch.empty(0, dtype=torch.int64, device=bc_mask.device)
    t = torch.tensor(ids, dtype=torch.uint8, device=bc_mask.device)
    return torch.nonzero(torch.isin(bc_mask.view(-1), t)).view(-1).to(torch.int64).contiguous()


class DifferentiableRun:
    """``num_steps`` steps of ``stepper`` as a differentiable function
    ``(f_init, aux_values) -> f_final``; call it like a function."""

    def __init__(self, stepper, bc_mask, missing_mask, omega, num_steps, checkpoint_every=100, use_graphs=True):
        pp = stepper.precision_policy
        if (pp.store_code, pp.compute_code) not in ((0, 0), (0, 1), (1, 1)):
            raise NotImplementedError(f"the adjoint supports FP32FP32, FP64FP32 and FP64FP64, not {pp}")
        if num_steps < 1 or checkpoint_every < 1:
            raise ValueError("num_steps and checkpoint_every must be >= 1")
        if bool((bc_mask == 255).any()):
            raise NotImplementedError("cells with id 255 are not differentiated (their populations are never rewritten)")
        self.stepper = stepper
        self.bc_mask = bc_mask
        self.missing_mask = missing_mask
        self.omega = float(omega)
        self.num_steps = int(num_steps)
        self.k = int(min(checkpoint_every, num_steps))
        self.bits = stepper._aux_state(bc_mask, missing_mask)[0]
        bcs = stepper.boundary_conditions
        kind = {bc.id: bc.kind for bc in bcs}
        # every boundary cell: the adjoint kernel runs their local adjoint in its second pass
        self.bc_cells = _cells_of(bc_mask, list(kind))
        self.aux_cells = _cells_of(bc_mask, [i for i, k in kind.items() if k in _AUX])
        # position of every aux cell inside bc_cells (both sorted)
        self.aux_pos = torch.searchsorted(self.bc_cells, self.aux_cells)
        self.store_dtype = pp.store_precision.torch_dtype
        self.compute_dtype = pp.compute_precision.torch_dtype
        self.state_shape = (stepper.velocity_set.q,) + tuple(stepper.grid.field_shape)
        self.n_cells = stepper.grid.num_cells
        self.peak_buffer_bytes = 0
        self.use_graphs = use_graphs
        self._graphs = {}
        self._states = None
        self._generation = 0

    def aux_from_fields(self, f_1):
        """The prescribed values as prepare_fields stored them (slot 0 of f_1)."""
        return f_1[0].reshape(-1)[self.aux_cells].to(self.compute_dtype)

    def __call__(self, f_init, aux_values=None):
        if aux_values is None:
            aux_values = torch.zeros(self.aux_cells.numel(), dtype=self.compute_dtype, device=f_init.device)
        return _Run.apply(f_init, aux_values, self)

    # ------------------------------------------------------------ C calls
    def _aux_field(self, aux_values):
        a = torch.zeros(self.n_cells, dtype=self.store_dtype, device=self.bc_mask.device)
        if self.aux_cells.numel():
            a[self.aux_cells] = aux_values.detach().to(self.store_dtype)
        return a

    def _forward(self, states, n, aux_field):
        lib = self.stepper._lib
        _lib.check(lib.xlbg_forward_segment(self.stepper.desc, _lib.ptr(states), int(n), _lib.ptr(self.bc_mask),
                                            _lib.ptr(self.bits), _lib.ptr(aux_field), self.omega,
                                            _lib.stream_handle()))

    def _adjoint(self, states, n, aux_field, lam_a, lam_b, aux_grad):
        lib = self.stepper._lib
        nbc = self.bc_cells.numel()
        _lib.check(lib.xlbg_adjoint_segment(
            self.stepper.desc, _lib.ptr(states), int(n), _lib.ptr(self.bc_mask), _lib.ptr(self.bits),
            _lib.ptr(aux_field), _lib.ptr(self.bc_cells) if nbc else None, nbc, _lib.ptr(lam_a), _lib.ptr(lam_b),
            _lib.ptr(aux_grad) if nbc else None, self.omega, _lib.stream_handle()))

    def segments(self):
        """(start step, steps) of each checkpoint segment."""
        nseg = math.ceil(self.num_steps / self.k)
        return [(s * self.k, min(self.k, self.num_steps - s * self.k)) for s in range(nseg)]

    # ------------------------------------------------------------ persistent buffers and graphs
    def _buffers(self, device):
        """The recorded segment, the aux field and the adjoint pair, owned by the plan
        so that captured graphs can replay on them."""
        if self._states is None:
            self._states = torch.empty((self.k + 1,) + self.state_shape, dtype=self.store_dtype, device=device)
            self._aux_buf = torch.zeros(self.n_cells, dtype=self.store_dtype, device=device)
            self._lam = [torch.empty(self.state_shape, dtype=self.compute_dtype, device=device) for _ in range(2)]
            self._aux_grad = torch.zeros(max(1, self.bc_cells.numel()), dtype=self.compute_dtype, device=device)
        return self._states

    def _run_graph(self, key, fn):
        """fn() once as a captured CUDA graph, replayed on later calls with the same
        key; direct calls if capture is unavailable."""
        if self.use_graphs:
            g = self._graphs.get(key)
            if g is None:
                try:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g):
                        fn()
                    self._graphs[key] = g
                except Exception:  # capture refused: run the same kernels directly from now on
                    self.use_graphs = False
                    self._graphs.clear()
                    torch.cuda.synchronize()
                    fn()
                    return
            g.replay()
            return
        fn()

    def _record(self, n):
        if n > 0:
            self._run_graph(("fwd", n), lambda: self._forward(self._states, n, self._aux_buf))

    def _reverse(self, n, swapped):
        lam_a, lam_b = (self._lam[1], self._lam[0]) if swapped else (self._lam[0], self._lam[1])
        self._run_graph(("adj", n, swapped),
                        lambda: self._adjoint(self._states, n, self._aux_buf, lam_a, lam_b, self._aux_grad))


class _Run(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f_init, aux_values, plan):
        if tuple(f_init.shape) != plan.state_shape or f_init.dtype != plan.store_dtype or not f_init.is_cuda:
            raise ValueError(f"f_init must be a CUDA {plan.store_dtype} tensor of shape {plan.state_shape}")
        states = plan._buffers(f_init.device)
        aux_field = plan._aux_field(aux_values)
        plan._aux_buf.copy_(aux_field)
        checkpoints = []
        cur = f_init.detach()
        for _, n in plan.segments():
            checkpoints.append(cur.clone())
            states[0].copy_(cur)
            plan._record(n)
            cur = states[n]
        out = cur.clone()
        plan._generation += 1
        ctx.generation = plan._generation
        ctx.plan = plan
        ctx.checkpoints = checkpoints
        ctx.aux_field = aux_field
        ctx.f_dtype = f_init.dtype
        ctx.aux_dtype = aux_values.dtype
        plan.peak_buffer_bytes = (states.numel() + sum(c.numel() for c in checkpoints)) * states.element_size()
        return out

    @staticmethod
    def backward(ctx, grad_out):
        plan = ctx.plan
        states = plan._states
        plan._aux_buf.copy_(ctx.aux_field)
        plan._lam[0].copy_(grad_out.detach())
        plan._aux_grad.zero_()
        # the recorded last segment is this call's only if no later forward overwrote it
        recorded = ctx.generation == plan._generation
        segs = plan.segments()
        swapped = False  # True: the current adjoint is in _lam[1]
        for i in range(len(segs) - 1, -1, -1):
            _, n = segs[i]
            if i != len(segs) - 1 or not recorded:
                states[0].copy_(ctx.checkpoints[i])
                plan._record(n - 1)
            plan._reverse(n, swapped)
            if n % 2:
                swapped = not swapped
        lam = plan._lam[1] if swapped else plan._lam[0]
        g_aux = plan._aux_grad[plan.aux_pos].to(ctx.aux_dtype) if plan.aux_cells.numel() else None
        plan._generation += 1  # the recorded segment now holds replayed states
        ctx.checkpoints = None
        return lam.to(ctx.f_dtype).clone(), g_aux, None
