from xlb_gb300.helper.check_boundary_overlaps import check_bc_overlaps
from xlb_gb300.helper.initializers import initialize_eq
from xlb_gb300.helper.nse_solver import create_nse_fields

__all__ = ["check_bc_overlaps", "initialize_eq", "create_nse_fields"]
