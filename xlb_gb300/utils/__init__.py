from xlb_gb300.utils.utils import save_fields_vtk, save_image

__all__ = ["save_fields_vtk", "save_image"]
