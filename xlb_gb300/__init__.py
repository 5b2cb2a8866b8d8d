"""GB300-native drop-in for XLB's fused lattice Boltzmann time step.

The import surface mirrors XLB's (xlb/__init__.py): ``init``, ``DefaultConfig``,
``ComputeBackend``, ``PrecisionPolicy``, ``Precision``, ``velocity_set``,
``grid``, ``operator`` (boundary conditions, stepper, macroscopic, equilibrium),
``helper`` and ``utils`` (field output).  Compute runs in hand-written sm_103a CUDA kernels in
``libxlbg.so``, called through a C ABI (include/xlbg.h).
"""

from xlb_gb300.compute_backend import ComputeBackend
from xlb_gb300.precision_policy import Precision, PrecisionPolicy
from xlb_gb300.default_config import DefaultConfig, init

import xlb_gb300.velocity_set as velocity_set  # noqa: E402
import xlb_gb300.grid as grid  # noqa: E402
import xlb_gb300.operator.boundary_condition  # noqa: E402,F401
import xlb_gb300.operator.stepper  # noqa: E402,F401
import xlb_gb300.operator.macroscopic  # noqa: E402,F401
import xlb_gb300.operator.equilibrium  # noqa: E402,F401
import xlb_gb300.helper as helper  # noqa: E402
import xlb_gb300.utils as utils  # noqa: E402

__version__ = "0.1.0"

__all__ = ["ComputeBackend", "Precision", "PrecisionPolicy", "DefaultConfig", "init", "velocity_set", "grid", "helper", "utils"]
