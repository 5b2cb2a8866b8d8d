from xlb_gb300.operator.boundary_masker.indices_boundary_masker import IndicesBoundaryMasker

__all__ = ["IndicesBoundaryMasker"]
