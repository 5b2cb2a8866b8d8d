"""The boundary conditions on the stepper's hot path.

Constructor signatures follow XLB's classes; the per-cell arithmetic is in the
fused CUDA step kernel (xlb_gb300/csrc/physics.cuh, step_kernel.cuh).

* FullwayBounceBackBC     collision step  (bc_fullway_bounce_back.py:22-86)
* HalfwayBounceBackBC     streaming step  (bc_halfway_bounce_back.py:22-99)
* EquilibriumBC           streaming step  (bc_equilibrium.py:24-101)
* ZouHeBC                 streaming step  (bc_zouhe.py:25-362)
* RegularizedBC           streaming step  (bc_regularized.py:21-220)
* ExtrapolationOutflowBC  streaming step  (bc_extrapolation_outflow.py:24-209)
"""

from collections import Counter

import numpy as np

from xlb_gb300 import _lib
from xlb_gb300.operator.boundary_condition.boundary_condition import BoundaryCondition, ImplementationStep


class FullwayBounceBackBC(BoundaryCondition):
    """f_out[l] = f_post_stream[opp l] at the BC cell."""

    kind = _lib.BC_FULLWAY_BB

    def __init__(self, velocity_set=None, precision_policy=None, compute_backend=None, indices=None, mesh_vertices=None):
        super().__init__(ImplementationStep.COLLISION, velocity_set, precision_policy, compute_backend, indices, mesh_vertices)


class HalfwayBounceBackBC(BoundaryCondition):
    """For missing l: f[l] = f_pre[opp l] (own-cell pre-stream value)."""

    kind = _lib.BC_HALFWAY_BB

    def __init__(self, velocity_set=None, precision_policy=None, compute_backend=None, indices=None, mesh_vertices=None):
        super().__init__(ImplementationStep.STREAMING, velocity_set, precision_policy, compute_backend, indices, mesh_vertices)
        self.needs_padding = True


class EquilibriumBC(BoundaryCondition):
    """f = feq(rho, u) with constant rho, u."""

    kind = _lib.BC_EQUILIBRIUM

    def __init__(
        self,
        rho: float,
        u,
        equilibrium_operator=None,
        velocity_set=None,
        precision_policy=None,
        compute_backend=None,
        indices=None,
        mesh_vertices=None,
    ):
        self.rho = float(rho)
        self.u = tuple(float(v) for v in u)
        self.equilibrium_operator = equilibrium_operator
        super().__init__(ImplementationStep.STREAMING, velocity_set, precision_policy, compute_backend, indices, mesh_vertices)
        if len(self.u) != self.velocity_set.d:
            raise ValueError(f"u must have {self.velocity_set.d} components")

    def c_entry(self):
        u = tuple(self.u) + (0.0,) * (3 - len(self.u))
        return (self.id, self.kind, self.rho, u)


class ZouHeBC(BoundaryCondition):
    """Zou-He velocity or pressure BC with non-equilibrium bounce-back.

    As in XLB's Warp path (bc_zouhe.py:96-100, :302-303) the prescribed value is
    one number: for ``"velocity"`` the single non-zero component of
    ``prescribed_value``, applied along the inward normal; for ``"pressure"``
    the density.  It is stored per cell in slot 0 of f_1 by ``aux_values``
    (boundary_condition.py:151-152).

    ``profile``, when given instead of ``prescribed_value``, is a callable that
    takes the BC cells' indices as an int array of shape (3, n) and returns n
    values (XLB takes a Warp function of one index).
    """

    _kinds = {"velocity": _lib.BC_ZOUHE_VELOCITY, "pressure": _lib.BC_ZOUHE_PRESSURE}

    def __init__(
        self,
        bc_type,
        profile=None,
        prescribed_value=None,
        velocity_set=None,
        precision_policy=None,
        compute_backend=None,
        indices=None,
        mesh_vertices=None,
    ):
        if bc_type not in ("velocity", "pressure"):
            raise ValueError(f"type = {bc_type} not supported! Use 'pressure' or 'velocity'.")
        self.bc_type = bc_type
        self.profile = profile
        super().__init__(ImplementationStep.STREAMING, velocity_set, precision_policy, compute_backend, indices, mesh_vertices)
        self.prescribed_value = None
        if prescribed_value is not None:
            if profile is not None:
                raise ValueError("Cannot specify both profile and prescribed_value")
            if isinstance(prescribed_value, (tuple, list)):
                prescribed_value = np.array(prescribed_value, dtype=np.float64)
            elif isinstance(prescribed_value, (int, float)):
                if bc_type == "pressure":
                    prescribed_value = float(prescribed_value)
                else:
                    raise ValueError("Velocity prescribed_value must be a tuple or array")
            elif isinstance(prescribed_value, np.ndarray):
                prescribed_value = prescribed_value.astype(np.float64)
            if bc_type == "velocity":
                if not isinstance(prescribed_value, np.ndarray):
                    raise ValueError("Velocity prescribed_value must be an array-like")
                if np.count_nonzero(prescribed_value) > 1:
                    raise ValueError("This BC only supports normal prescribed values (only one non-zero element allowed)")
                nz = np.nonzero(prescribed_value)[0]
                prescribed_value = float(prescribed_value[nz][0]) if nz.size else 0.0
            self.prescribed_value = float(prescribed_value)
        elif profile is None:
            raise ValueError("ZouHe / Regularized BCs need a profile or a prescribed_value")
        self.needs_aux_init = True
        self.needs_aux_recovery = True
        self.num_of_aux_data = 1
        self.needs_padding = True

    @property
    def kind(self):
        return self._kinds[self.bc_type]

    def aux_values(self, cell_indices):
        """Prescribed value at each BC cell; cell_indices is (3, n) int64."""
        n = cell_indices.shape[1]
        if self.profile is not None:
            vals = self.profile(cell_indices)
            if hasattr(vals, "detach"):
                vals = vals.detach().cpu().numpy()
            vals = np.asarray(vals, dtype=np.float64).reshape(-1)
            if vals.size == 1 and n != 1:
                vals = np.full(n, float(vals[0]))
            if vals.size != n:
                raise ValueError(f"profile returned {vals.size} values for {n} cells")
            return vals
        return np.full(n, self.prescribed_value, dtype=np.float64)


class RegularizedBC(ZouHeBC):
    """ZouHe followed by regularisation f = feq + 4.5 w (Qi : Pi_neq)."""

    _kinds = {"velocity": _lib.BC_REGULARIZED_VELOCITY, "pressure": _lib.BC_REGULARIZED_PRESSURE}


class ExtrapolationOutflowBC(BoundaryCondition):
    """Outflow: streaming step bounces the stored extrapolated values back in;
    after collision the outgoing slots receive (1-cs) f_ps[l] + cs f_ps_neighbour[l]."""

    kind = _lib.BC_EXTRAPOLATION

    def __init__(self, velocity_set=None, precision_policy=None, compute_backend=None, indices=None, mesh_vertices=None):
        super().__init__(ImplementationStep.STREAMING, velocity_set, precision_policy, compute_backend, indices, mesh_vertices)
        self.normal = self._get_normal_vec(indices) if indices is not None else None

    @staticmethod
    def _get_normal_vec(indices):
        """Global normal from the index set (bc_extrapolation_outflow.py:283-297).
        Kept for API parity; the kernel uses the per-cell normal, as XLB's Warp path does."""
        freq = [Counter(np.asarray(coord).reshape(-1).tolist()).most_common(1)[0] for coord in indices]
        counts = np.array([c for _, c in freq])
        elements = np.array([e for e, _ in freq])
        normal = counts // counts.max()
        if elements[np.argmax(counts)] == 0:
            normal = normal * -1
        return normal
