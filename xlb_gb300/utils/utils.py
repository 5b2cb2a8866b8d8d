"""Field output after the step: legacy VTK files and PNG images.

Same names and arguments as XLB's xlb/utils/utils.py:50-146 (``save_image``,
``save_fields_vtk``), for fields read out of the populations with the
macroscopic operator.  XLB writes through pyvista and matplotlib; neither is
needed here: the VTK file is the legacy binary format written directly (what
pyvista's ``ImageData.save(..., binary=True)`` produces for a ``.vtk`` name:
cell data on a uniform grid with unit spacing) and the PNG is an 8-bit
grayscale image written with zlib.  Fields may be numpy arrays or torch tensors
(on any device).
"""

import os
import struct
import time
import zlib

import numpy as np


def _to_numpy(a):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a)


def save_fields_vtk(fields, timestep, output_dir=".", prefix="fields"):
    """Write ``fields`` (name -> array of shape (nx, ny) or (nx, ny, nz), all the
    same shape) as cell data of one uniform grid to
    ``<output_dir>/<prefix>_<timestep:07d>.vtk`` (xlb/utils/utils.py:93-146).
    float32 fields are written as float, everything else as double."""
    arrays = {k: _to_numpy(v) for k, v in fields.items()}
    if not arrays:
        raise ValueError("no fields to save")
    shape = next(iter(arrays.values())).shape
    for k, v in arrays.items():
        if v.shape != shape:
            raise AssertionError("All fields must have the same dimensions!")
    if len(shape) not in (2, 3):
        raise ValueError("fields must be 2D (nx, ny) or 3D (nx, ny, nz)")
    dims = tuple(d + 1 for d in shape) + ((1,) if len(shape) == 2 else ())  # points = cells + 1
    ncell = int(np.prod(shape))
    path = os.path.join(output_dir, f"{prefix}_{timestep:07d}.vtk")
    start = time.time()
    with open(path, "wb") as fh:
        fh.write(b"# vtk DataFile Version 3.0\n")
        fh.write(b"xlb_gb300 fields\nBINARY\nDATASET STRUCTURED_POINTS\n")
        fh.write(f"DIMENSIONS {dims[0]} {dims[1]} {dims[2]}\n".encode())
        fh.write(b"ORIGIN 0 0 0\nSPACING 1 1 1\n")
        fh.write(f"CELL_DATA {ncell}\n".encode())
        for name, v in arrays.items():
            kind, be = ("float", ">f4") if v.dtype == np.float32 else ("double", ">f8")
            fh.write(f"SCALARS {name} {kind} 1\nLOOKUP_TABLE default\n".encode())
            # VTK's point / cell order has x fastest: Fortran order of (nx, ny[, nz])
            fh.write(np.ascontiguousarray(v.flatten(order="F").astype(be)).tobytes())
            fh.write(b"\n")
    print(f"Saved {path} in {time.time() - start:.6f} seconds.")
    return path


def _png(path, gray):
    """8-bit grayscale PNG (rows top to bottom)."""
    h, w = gray.shape

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    raw = b"".join(b"\x00" + gray[r].tobytes() for r in range(h))  # filter type 0 per row
    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n")
        fh.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)))
        fh.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        fh.write(chunk(b"IEND", b""))


def save_image(fld, timestep=None, prefix=None, **kwargs):
    """Save a 2D field as ``<prefix>[_<timestep:04d>].png`` (xlb/utils/utils.py:50-90):
    x to the right, y up (XLB plots ``fld.T`` with origin 'lower').  A field of
    shape (c, nx, ny) is shown as its magnitude over the components (XLB's code
    squares component 0 twice there).  The image is grayscale, min to max; XLB's
    matplotlib colormap is not reproduced.  ``vmin`` / ``vmax`` fix the range."""
    if prefix is None:
        import __main__

        fname = os.path.splitext(os.path.basename(getattr(__main__, "__file__", "field")))[0]
    else:
        fname = prefix
    if timestep is not None:
        fname = fname + "_" + str(timestep).zfill(4)
    f = _to_numpy(fld).astype(np.float64)
    if f.ndim > 3:
        raise ValueError("The input field should be 2D!")
    if f.ndim == 3:
        f = np.sqrt((f**2).sum(axis=0))
    lo = kwargs.get("vmin", np.nanmin(f))
    hi = kwargs.get("vmax", np.nanmax(f))
    scale = 255.0 / (hi - lo) if hi > lo else 0.0
    g = np.clip(np.nan_to_num((f - lo) * scale), 0, 255).astype(np.uint8)
    img = np.ascontiguousarray(g.T[::-1])  # rows: y from top (ny-1) to bottom (0); columns: x
    path = fname + ".png"
    _png(path, img)
    return path
