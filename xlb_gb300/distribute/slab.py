"""Slab decomposition of the fused step along x.

XLB's only parallel strategy shards the grid along array axis 1 (x, the slowest
spatial axis) and, after each step on a shard, moves the x-crossing populations
of the first and last x-planes to the neighbouring shards with a pair of
``ppermute`` calls (xlb/distribute/distribute.py:10-105,
xlb/operator/parallel_operator.py:6-82; the crossing sets are
velocity_set.py:199-221, ``right_indices`` / ``left_indices``).

Here a slab of t x-planes is held with one ghost plane on each side, as a
field of shape (Q, t + 2, ...) whose ghost planes are marked 255 in bc_mask (the
step kernel skips them) and are filled before every step:

- left ghost  <- the left neighbour's last interior plane, directions with c_x = +1,
- right ghost <- the right neighbour's first interior plane, directions with c_x = -1,

with the periodic wrap of the stream between the first and last slab.  Those
are the only values a pull of an interior cell reads outside its slab (the
extrapolation outflow's neighbour read stays within one plane as well), so the
interior cells of every slab compute exactly what the single-domain step
computes: results are bit-identical.  Per step and slab the exchange moves
2 x |crossing| x ny x nz values: 5 of 19 (D3Q19), 9 of 27 (D3Q27), 3 of 9 (D2Q9).

Transports:

- ``LocalTransport``: every slab lives in this process (one GPU, or several
  devices of this process); ghost planes are device-local copies.
- ``ProcessGroupTransport``: one slab per rank of a torch.distributed process
  group; ghost planes travel as point-to-point messages (NCCL between GPUs,
  gloo between CPU processes), the equivalent of XLB's two ppermutes.

Diagnostics (mass of the new state, momentum-exchange force) are summed per
slab in FP64 by the fused diagnostics step and then over slabs in FP64 (an
all-reduce for the process-group transport).  The exchange is issued before
the step kernels rather than overlapped with the interior: at 512 x 512 x 512
cells per slab it moves 2 x 5 MB against 20 GB of step traffic.
"""

import numpy as np
import torch

from xlb_gb300 import _lib


class SlabLayout:
    """x-ranges [x0, x1) of n slabs over nx cells: near-equal thickness, the
    first nx mod n slabs one plane thicker (XLB requires nx divisible by the
    device count; uneven splits are allowed here)."""

    def __init__(self, nx, n_slabs):
        nx, n_slabs = int(nx), int(n_slabs)
        if n_slabs < 1 or n_slabs > nx:
            raise ValueError(f"cannot split {nx} x-planes into {n_slabs} slabs")
        base, extra = divmod(nx, n_slabs)
        self.nx = nx
        self.n = n_slabs
        self.bounds = []
        x = 0
        for r in range(n_slabs):
            t = base + (1 if r < extra else 0)
            self.bounds.append((x, x + t))
            x += t

    def thickness(self, r):
        x0, x1 = self.bounds[r]
        return x1 - x0

    def padded_planes(self, r):
        """Global x of each plane of slab r's padded field (ghosts included, periodic)."""
        x0, x1 = self.bounds[r]
        return [(x0 - 1 + p) % self.nx for p in range(x1 - x0 + 2)]


def crossing_directions(velocity_set):
    """(right, left): directions with c_x = +1 (read from the left neighbour)
    and with c_x = -1 (read from the right neighbour), in direction order
    (velocity_set.py:199-221)."""
    c = np.asarray(velocity_set.c)
    right = [l for l in range(velocity_set.q) if c[0, l] == 1]
    left = [l for l in range(velocity_set.q) if c[0, l] == -1]
    return right, left


class SlabFields:
    """One slab's padded fields and its per-slab step state."""

    def __init__(self, index, x0, x1, f_0, f_1, bc_mask, missing_mask):
        self.index = index
        self.x0, self.x1 = x0, x1
        self.t = x1 - x0
        self.f_0, self.f_1 = f_0, f_1
        self.bc_mask, self.missing_mask = bc_mask, missing_mask
        self.bits = self.rec = self.scratch = None
        self.desc = None
        self.diag_slots = None

    @property
    def device(self):
        return self.f_0.device

    def swap(self):
        self.f_0, self.f_1 = self.f_1, self.f_0


def _as_slice(dirs):
    """The direction list as a slice when it is an arithmetic progression (it is
    for XLB's orderings: D3Q19 14..18 / 9..13, D3Q27 18..26 / 9..17, D2Q9 3,5,7 /
    4,6,8), else None."""
    if len(dirs) == 1:
        return slice(dirs[0], dirs[0] + 1)
    step = dirs[1] - dirs[0]
    if step > 0 and all(b - a == step for a, b in zip(dirs, dirs[1:])):
        return slice(dirs[0], dirs[-1] + 1, step)
    return None


def _plane_copy(dst, dst_plane, src, src_plane, dirs):
    """dst[dirs, dst_plane] = src[dirs, src_plane]: one strided copy when the
    directions are evenly spaced, else one copy per direction (each (l, plane)
    block is contiguous in the (Q, x, ...) layout)."""
    sl = _as_slice(dirs)
    if sl is not None:
        dst[sl, dst_plane].copy_(src[sl, src_plane], non_blocking=True)
        return
    for l in dirs:
        dst[l, dst_plane].copy_(src[l, src_plane], non_blocking=True)


class LocalTransport:
    """All slabs in this process: ghost planes by device-local copies."""

    size = 1
    rank = 0

    def local_slab_indices(self, n_slabs):
        return list(range(n_slabs))

    def exchange(self, slabs, right, left, n_slabs):
        if len(slabs) != n_slabs:
            raise ValueError("LocalTransport needs every slab in this process")
        for r, s in enumerate(slabs):
            lft = slabs[(r - 1) % n_slabs]
            rgt = slabs[(r + 1) % n_slabs]
            _plane_copy(s.f_0, 0, lft.f_0, lft.t, right)
            _plane_copy(s.f_0, s.t + 1, rgt.f_0, 1, left)

    def all_reduce(self, t):
        return t


class ProcessGroupTransport:
    """One slab per rank: ghost planes as point-to-point messages of a
    torch.distributed process group (NCCL for GPUs, gloo for CPU tensors).
    Rank r sends its last interior plane's c_x = +1 values to rank r + 1 and its
    first interior plane's c_x = -1 values to rank r - 1 (periodic), and
    receives the mirror pair: XLB's rightPerm / leftPerm ppermutes
    (distribute.py:21-44)."""

    def __init__(self, group=None):
        import torch.distributed as dist

        if not dist.is_initialized():
            raise RuntimeError("ProcessGroupTransport needs an initialised torch.distributed process group")
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)

    def local_slab_indices(self, n_slabs):
        if n_slabs != self.size:
            raise ValueError(f"{n_slabs} slabs over {self.size} ranks: one slab per rank")
        return [self.rank]

    def exchange(self, slabs, right, left, n_slabs):
        (s,) = slabs
        if self.size == 1:
            _plane_copy(s.f_0, 0, s.f_0, s.t, right)
            _plane_copy(s.f_0, s.t + 1, s.f_0, 1, left)
            return
        dist = self.dist
        sr, sl = _as_slice(right), _as_slice(left)
        send_r = s.f_0[sr, s.t].contiguous() if sr is not None else torch.stack([s.f_0[l, s.t] for l in right])
        send_l = s.f_0[sl, 1].contiguous() if sl is not None else torch.stack([s.f_0[l, 1] for l in left])
        recv_l = torch.empty_like(send_r)
        recv_r = torch.empty_like(send_l)
        prev = dist.get_global_rank(self.group, (self.rank - 1) % self.size) if self.group else (self.rank - 1) % self.size
        nxt = dist.get_global_rank(self.group, (self.rank + 1) % self.size) if self.group else (self.rank + 1) % self.size
        ops = [
            dist.P2POp(dist.isend, send_r, nxt, self.group, 0),
            dist.P2POp(dist.irecv, recv_l, prev, self.group, 0),
            dist.P2POp(dist.isend, send_l, prev, self.group, 1),
            dist.P2POp(dist.irecv, recv_r, nxt, self.group, 1),
        ]
        for req in dist.batch_isend_irecv(ops):
            req.wait()
        if sr is not None:
            s.f_0[sr, 0].copy_(recv_l)
        else:
            for k, l in enumerate(right):
                s.f_0[l, 0].copy_(recv_l[k])
        if sl is not None:
            s.f_0[sl, s.t + 1].copy_(recv_r)
        else:
            for k, l in enumerate(left):
                s.f_0[l, s.t + 1].copy_(recv_r[k])

    def all_reduce(self, t):
        self.dist.all_reduce(t, group=self.group)
        return t


def _default_transport():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        return ProcessGroupTransport()
    return LocalTransport()


class DistributedStepper:
    """The stepper run over x-slabs (the counterpart of XLB's
    ``distribute(stepper, grid, velocity_set)``, distribute.py:85-105).

        dstep = DistributedStepper(stepper, n_slabs=2)
        slabs = dstep.scatter(f_0, f_1, bc_mask, missing_mask)   # or dstep.prepare_fields()
        for i in range(n):
            slabs = dstep(slabs, omega, i)                       # exchange + step + swap
        f_0, f_1 = dstep.gather(slabs)

    Each call fills the ghost planes of every local slab's f_0, runs the fused
    step on every local slab (``xlbg_step`` with a per-slab descriptor) and
    swaps the slab's buffers, so ``slab.f_0`` holds the newest state, as XLB's
    loop holds it after its swap.  ``local_step(slab, omega, timestep)`` replaces
    the per-slab step (used to run the schedule with a CPU step in tests)."""

    def __init__(self, stepper, n_slabs=None, transport=None, local_step=None):
        self.stepper = stepper
        self.velocity_set = stepper.velocity_set
        self.transport = transport if transport is not None else _default_transport()
        if n_slabs is None:
            n_slabs = self.transport.size if isinstance(self.transport, ProcessGroupTransport) else 1
        self.layout = SlabLayout(stepper.grid.shape[0], n_slabs)
        self.local = self.transport.local_slab_indices(n_slabs)
        self.right, self.left = crossing_directions(self.velocity_set)
        self.local_step = local_step
        self._rec_ids = [bc.id for bc in stepper.boundary_conditions if bc.needs_aux_recovery]

    # ------------------------------------------------------------------ fields

    def _slab_from_global(self, r, f_0, f_1, bc_mask, missing_mask, device):
        planes = torch.tensor(self.layout.padded_planes(r), dtype=torch.long, device=f_0.device)
        x0, x1 = self.layout.bounds[r]
        take = lambda a: a.index_select(1, planes.to(a.device)).to(device).contiguous()  # noqa: E731
        bm = take(bc_mask)
        bm[:, 0] = 255
        bm[:, -1] = 255
        mm = take(missing_mask)
        mm[:, 0] = False
        mm[:, -1] = False
        return SlabFields(r, x0, x1, take(f_0), take(f_1), bm, mm)

    def scatter(self, f_0, f_1, bc_mask, missing_mask, device=None):
        """The local slabs of global fields (any device; slabs go to ``device``,
        default the fields' device)."""
        dev = torch.device(device) if device is not None else f_0.device
        return [self._slab_from_global(r, f_0, f_1, bc_mask, missing_mask, dev) for r in self.local]

    def prepare_fields(self, device=None):
        """The local slabs of the stepper's prepare_fields() without global
        populations: the masks are built for the whole grid (XLB's maskers need
        the global bounds) on ``device`` (default: the current CUDA device),
        sliced and released; each slab's f_0 is the rest equilibrium and its
        f_1 a copy carrying the ZouHe / Regularized aux values of its cells
        (boundary_condition.py:130-159, evaluated at global indices)."""
        from xlb_gb300.helper.initializers import initialize_eq

        st = self.stepper
        vs = st.velocity_set
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        fs = tuple(st.grid.field_shape)
        bc_mask = torch.zeros((1,) + fs, dtype=torch.uint8, device=dev)
        missing = torch.zeros((vs.q,) + fs, dtype=torch.bool, device=dev)
        bc_mask, missing = st._process_boundary_conditions(st.boundary_conditions, bc_mask, missing)
        cdt = st.precision_policy.compute_precision.torch_dtype
        slabs = []
        for r in self.local:
            planes = torch.tensor(self.layout.padded_planes(r), dtype=torch.long, device=dev)
            x0, x1 = self.layout.bounds[r]
            bm = bc_mask.index_select(1, planes).contiguous()
            bm[:, 0] = 255
            bm[:, -1] = 255
            mm = missing.index_select(1, planes).contiguous()
            mm[:, 0] = False
            mm[:, -1] = False
            f_0 = torch.empty((vs.q,) + tuple(bm.shape[1:]), dtype=st.store_dtype, device=dev)
            f_0 = initialize_eq(f_0, None, vs, st.precision_policy)
            f_1 = f_0.clone()
            for bc in st.boundary_conditions:
                if not bc.needs_aux_init:
                    continue
                lin = torch.nonzero(bm.view(-1) == bc.id).view(-1)
                if lin.numel() == 0:
                    continue
                idx = np.array(np.unravel_index(lin.cpu().numpy(), tuple(bm.shape[1:])))
                idx[0] = (x0 - 1 + idx[0]) % self.layout.nx  # padded plane -> global x
                vals = torch.as_tensor(bc.aux_values(idx), dtype=torch.float64, device=dev)
                f_1[0].view(-1)[lin] = vals.to(cdt).to(f_1.dtype)
            slabs.append(SlabFields(r, x0, x1, f_0, f_1, bm, mm))
        del bc_mask, missing
        return slabs

    def gather(self, slabs):
        """Global (f_0, f_1) from every slab (all slabs must be local)."""
        if len(slabs) != self.layout.n:
            raise ValueError("gather needs every slab in this process")
        f_0 = torch.cat([s.f_0[:, 1 : s.t + 1] for s in slabs], dim=1)
        f_1 = torch.cat([s.f_1[:, 1 : s.t + 1] for s in slabs], dim=1)
        return f_0, f_1

    # ------------------------------------------------------------------ stepping

    def _slab_state(self, s):
        if s.desc is None:
            d = _lib.Desc.from_buffer_copy(self.stepper.desc)
            d.nx = s.t + 2
            s.desc = d
            lib = _lib.load()
            n = s.bc_mask.numel()
            with torch.cuda.device(s.device):
                s.bits = torch.empty(n, dtype=torch.int32, device=s.device)
                _lib.check(lib.xlbg_pack_missing(d, _lib.ptr(s.missing_mask), _lib.ptr(s.bits), _lib.stream_handle()))
                if self._rec_ids:
                    ids = torch.tensor(self._rec_ids, dtype=torch.uint8, device=s.device)
                    s.rec = torch.nonzero(torch.isin(s.bc_mask.view(-1), ids)).view(-1).to(torch.int64).contiguous()
                    s.scratch = torch.empty(max(1, s.rec.numel()) * self.velocity_set.q, dtype=s.f_0.dtype,
                                            device=s.device)
        return s

    def _rec_args(self, s):
        if s.rec is None or s.rec.numel() == 0:
            return None, 0, None
        return _lib.ptr(s.rec), s.rec.numel(), _lib.ptr(s.scratch)

    def _step_slab(self, s, omega, timestep):
        self._slab_state(s)
        rc, nrec, scr = self._rec_args(s)
        with torch.cuda.device(s.device):
            _lib.check(_lib.load().xlbg_step(
                s.desc, _lib.ptr(s.f_0), _lib.ptr(s.f_1), _lib.ptr(s.bc_mask), _lib.ptr(s.bits), rc, nrec, scr,
                float(omega), int(timestep), _lib.stream_handle()))

    def __call__(self, slabs, omega, timestep):
        self.transport.exchange(slabs, self.right, self.left, self.layout.n)
        for s in slabs:
            if self.local_step is not None:
                self.local_step(s, omega, timestep)
            else:
                self._step_slab(s, omega, timestep)
            s.swap()
        return slabs

    def run(self, slabs, omega, num_steps, timestep0=0):
        for i in range(num_steps):
            self(slabs, omega, timestep0 + i)
        return slabs

    def step_with_diagnostics(self, slabs, omega, timestep, force_bc=None):
        """One step (exchange, step, swap) that also returns a float64 tensor of 4
        values on the first slab's device: [mass of the new state, force on
        ``force_bc`` (x, y[, z]) on the input state], each summed in FP64 over
        the slab's cells and then over all slabs (all-reduce across ranks)."""
        if self.local_step is not None:
            raise ValueError("diagnostics need the CUDA step")
        self.transport.exchange(slabs, self.right, self.left, self.layout.n)
        force_id = -1 if force_bc is None else int(force_bc.id)
        lib = _lib.load()
        total = None
        for s in slabs:
            self._slab_state(s)
            rc, nrec, scr = self._rec_args(s)
            with torch.cuda.device(s.device):
                if s.diag_slots is None:
                    s.diag_slots = torch.zeros(_lib.DIAG_SLOTS * 4, dtype=torch.float64, device=s.device)
                out = torch.empty(4, dtype=torch.float64, device=s.device)
                _lib.check(lib.xlbg_step_diag(
                    s.desc, _lib.ptr(s.f_0), _lib.ptr(s.f_1), _lib.ptr(s.bc_mask), _lib.ptr(s.bits), rc, nrec, scr,
                    float(omega), int(timestep), force_id, _lib.ptr(s.diag_slots), _lib.ptr(out),
                    _lib.stream_handle()))
            s.swap()
            total = out if total is None else total + out.to(total.device)
        return self.transport.all_reduce(total)


def distribute(operator, grid=None, velocity_set=None, n_slabs=None, transport=None):
    """XLB's ``distribute(stepper, grid, velocity_set)`` (distribute.py:85-105)
    for the stepper: a ``DistributedStepper`` over x-slabs."""
    from xlb_gb300.operator.stepper import IncompressibleNavierStokesStepper

    if not isinstance(operator, IncompressibleNavierStokesStepper):
        raise NotImplementedError("only the stepper is distributed on this path")
    return DistributedStepper(operator, n_slabs=n_slabs, transport=transport)


__all__ = ["SlabLayout", "SlabFields", "LocalTransport", "ProcessGroupTransport", "DistributedStepper",
           "crossing_directions", "distribute"]
