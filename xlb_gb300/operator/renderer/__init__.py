from xlb_gb300.operator.renderer.mesh_renderer import Mesh, MeshRenderer

__all__ = ["Mesh", "MeshRenderer"]
