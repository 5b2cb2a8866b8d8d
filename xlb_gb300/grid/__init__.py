from xlb_gb300.grid.grid import grid_factory, Grid, WarpGrid, CudaGrid

__all__ = ["grid_factory", "Grid", "WarpGrid", "CudaGrid"]
