from xlb_gb300.operator.boundary_condition.boundary_condition import (
    BoundaryCondition,
    BoundaryConditionRegistry,
    ImplementationStep,
    boundary_condition_registry,
)
from xlb_gb300.operator.boundary_condition.bc import (
    EquilibriumBC,
    ExtrapolationOutflowBC,
    FullwayBounceBackBC,
    HalfwayBounceBackBC,
    RegularizedBC,
    ZouHeBC,
)

__all__ = [
    "BoundaryCondition",
    "BoundaryConditionRegistry",
    "ImplementationStep",
    "boundary_condition_registry",
    "EquilibriumBC",
    "ExtrapolationOutflowBC",
    "FullwayBounceBackBC",
    "HalfwayBounceBackBC",
    "RegularizedBC",
    "ZouHeBC",
]
