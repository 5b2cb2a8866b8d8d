from xlb_gb300.operator.stepper.adjoint import DifferentiableRun
from xlb_gb300.operator.stepper.nse_stepper import IncompressibleNavierStokesStepper, Stepper

__all__ = ["IncompressibleNavierStokesStepper", "Stepper", "DifferentiableRun"]
