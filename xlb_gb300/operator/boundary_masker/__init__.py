from xlb_gb300.operator.boundary_masker.indices_boundary_masker import IndicesBoundaryMasker
from xlb_gb300.operator.boundary_masker.mesh_boundary_masker import MeshBoundaryMasker

__all__ = ["IndicesBoundaryMasker", "MeshBoundaryMasker"]
