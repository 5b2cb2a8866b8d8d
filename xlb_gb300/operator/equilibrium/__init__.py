from xlb_gb300.operator.equilibrium.quadratic_equilibrium import Equilibrium, QuadraticEquilibrium

__all__ = ["Equilibrium", "QuadraticEquilibrium"]
