from xlb_gb300.velocity_set.velocity_set import VelocitySet, D2Q9, D3Q19, D3Q27, lattice_code

__all__ = ["VelocitySet", "D2Q9", "D3Q19", "D3Q27", "lattice_code"]
