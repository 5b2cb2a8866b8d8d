"""Build the C-ABI descriptor (``xlbg_desc``) from XLB-style objects."""

from xlb_gb300 import _lib
from xlb_gb300.velocity_set import lattice_code


def spatial_shape(velocity_set, field_shape):
    """(nx, ny, nz) from a field's spatial shape; 2D fields carry nz = 1."""
    if velocity_set.d == 2:
        if len(field_shape) == 3 and field_shape[2] != 1:
            raise ValueError("2D fields have shape (q, nx, ny, 1)")
        return int(field_shape[0]), int(field_shape[1]), 1
    if len(field_shape) != 3:
        raise ValueError("3D fields have shape (q, nx, ny, nz)")
    return tuple(int(s) for s in field_shape)


def make_desc(velocity_set, precision_policy, shape3, collision=_lib.BGK, bcs=()):
    d = _lib.Desc()
    d.abi_version = _lib.ABI_VERSION
    d.lattice = lattice_code(velocity_set)
    d.store = precision_policy.store_code
    d.compute = precision_policy.compute_code
    d.collision = collision
    d.nx, d.ny, d.nz = shape3
    entries = [bc.c_entry() for bc in bcs]
    if len(entries) > _lib.MAX_BC:
        raise ValueError(f"at most {_lib.MAX_BC} boundary conditions per stepper")
    d.nbc = len(entries)
    for i, (bid, kind, rho, u) in enumerate(entries):
        d.bc[i].id = bid
        d.bc[i].kind = kind
        d.bc[i].rho = rho
        for k in range(3):
            d.bc[i].u[k] = u[k]
    return d
