"""Equilibrium initialisation (xlb/helper/initializers.py:5-20)."""

from xlb_gb300.operator.equilibrium import QuadraticEquilibrium


def initialize_eq(f, grid, velocity_set, precision_policy, compute_backend=None, rho=None, u=None):
    """f = feq(rho, u) in the store form; rho = 1 and u = 0 when not given."""
    eq = QuadraticEquilibrium(velocity_set, precision_policy)
    return eq(rho, u, f)
