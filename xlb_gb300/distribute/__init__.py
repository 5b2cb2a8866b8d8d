"""Slab decomposition of the stepper along x (XLB's xlb/distribute)."""

from xlb_gb300.distribute.slab import (
    DistributedStepper,
    LocalTransport,
    ProcessGroupTransport,
    SlabFields,
    SlabLayout,
    crossing_directions,
    distribute,
)

__all__ = ["DistributedStepper", "LocalTransport", "ProcessGroupTransport", "SlabFields", "SlabLayout",
           "crossing_directions", "distribute"]
