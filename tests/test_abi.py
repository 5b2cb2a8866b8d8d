"""libxlbg.so loads, exports every entry point include/xlbg.h declares, and
rejects bad descriptors on the host (no GPU work is launched by these calls)."""

import ctypes
import os
import re

import numpy as np
import pytest

import xlb_gb300 as xlb
from xlb_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(xlbg_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof / offsetof of the C structs (gcc on include/xlbg.h) equal the ctypes mirrors."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        "#include <stdio.h>\n#include <stddef.h>\n#include \"xlbg.h\"\n"
        "int main(void) { printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(xlbg_desc), offsetof(xlbg_desc, bc),"
        " sizeof(xlbg_bc), sizeof(xlbg_tri_grid), offsetof(xlbg_tri_grid, cell_start), sizeof(xlbg_camera),"
        " offsetof(xlbg_camera, gamma)); return 0; }\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(_lib.Desc), _lib.Desc.bc.offset, ctypes.sizeof(_lib.BCEntry), ctypes.sizeof(_lib.TriGrid),
            _lib.TriGrid.cell_start.offset, ctypes.sizeof(_lib.Camera), _lib.Camera.gamma.offset]
    assert got == want


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 9
    for n in names:
        assert hasattr(lib, n), n
    assert set(_lib.EXPORTED) <= set(names)
    assert lib.xlbg_abi_version() == _lib.ABI_VERSION


@pytest.mark.parametrize("code,cls", [(0, xlb.velocity_set.D2Q9), (1, xlb.velocity_set.D3Q19), (2, xlb.velocity_set.D3Q27)])
def test_compiled_lattice_tables_match_velocity_sets(code, cls):
    vs = cls()
    c, w, opp = _lib.lattice_tables(code)
    assert np.array_equal(c.T, vs.c)
    assert np.array_equal(w, vs.w)  # bit-identical doubles
    assert np.array_equal(opp, vs.opp_indices)


def _desc(**kw):
    d = _lib.Desc()
    d.abi_version = _lib.ABI_VERSION
    d.lattice, d.store, d.compute, d.collision, d.nbc = 1, 0, 0, 0, 0
    d.nx = d.ny = d.nz = 8
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _step(desc, f0=1024, f1=2048):
    lib = _lib.load()
    p = ctypes.c_void_p
    return lib.xlbg_step(desc, p(f0), p(f1), p(4096), p(8192), None, 0, None, 1.0, 0, None)


def test_null_and_bad_descriptors_are_rejected():
    lib = _lib.load()
    p = ctypes.c_void_p
    assert lib.xlbg_step(None, p(16), p(32), p(64), p(128), None, 0, None, 1.0, 0, None) == _lib.ERR_ARG
    assert b"NULL" in lib.xlbg_last_error()
    assert _step(_desc(abi_version=99)) == _lib.ERR_ARG
    assert _step(_desc(lattice=7)) == _lib.ERR_ARG
    assert _step(_desc(collision=_lib.KBC)) == _lib.ERR_UNSUPPORTED
    assert b"D2Q9 and D3Q27" in lib.xlbg_last_error()
    assert _step(_desc(compute=1, store=3)) == _lib.ERR_UNSUPPORTED
    assert _step(_desc(lattice=0, nz=4)) == _lib.ERR_ARG
    assert _step(_desc(nx=0)) == _lib.ERR_ARG
    d = _desc(nbc=1)
    d.bc[0].id, d.bc[0].kind = 255, _lib.BC_FULLWAY_BB
    assert _step(d) == _lib.ERR_ARG


def test_pointer_checks():
    assert _step(_desc(), f0=1026) == _lib.ERR_ALIGN
    assert _step(_desc(), f0=1024, f1=1024) == _lib.ERR_ARG
    lib = _lib.load()
    p = ctypes.c_void_p
    # n_rec > 0 needs both the cell list and the scratch
    assert lib.xlbg_step(_desc(), p(1024), p(2048), p(4096), p(8192), None, 5, None, 1.0, 0, None) == _lib.ERR_ARG


def test_xlbg_error_carries_message():
    with pytest.raises(_lib.XlbgError) as e:
        _lib.check(_step(_desc(collision=_lib.KBC)))
    assert e.value.code == _lib.ERR_UNSUPPORTED


def test_masker_and_renderer_entries_reject_bad_arguments():
    """Host-side checks of xlbg_indices_mask, xlbg_mesh_mask and xlbg_render_mesh
    (each returns before any CUDA call)."""
    lib = _lib.load()
    p = ctypes.c_void_p
    d = _desc()
    # indices masker: bad id, negative count, misaligned index array, 2D grid with nz != 1
    assert lib.xlbg_indices_mask(d, p(1024), 4, 0, 0, p(4096), p(8192), None) == _lib.ERR_ARG
    assert lib.xlbg_indices_mask(d, p(1024), -1, 3, 0, p(4096), p(8192), None) == _lib.ERR_ARG
    assert lib.xlbg_indices_mask(d, p(1028), 4, 3, 0, p(4096), p(8192), None) == _lib.ERR_ALIGN
    assert lib.xlbg_indices_mask(_desc(lattice=0, nz=2), p(1024), 4, 3, 0, p(4096), p(8192), None) == _lib.ERR_ARG
    assert lib.xlbg_indices_mask(d, p(1024), 0, 3, 0, None, None, None) == _lib.OK  # nothing to do
    # mesh masker: 2D lattice, unknown flag, bad brick, unaligned scratch
    args = dict(tri=p(1024), n=12, pt=p(2048), pb=p(4096), npairs=12, brick=8, bid=4, flags=0, rec=p(8192),
                solid=p(16384), bm=p(32768), mm=p(65536))

    def mesh(desc, **kw):
        a = dict(args, **kw)
        return lib.xlbg_mesh_mask(desc, a["tri"], a["n"], a["pt"], a["pb"], a["npairs"], a["brick"], a["bid"],
                                  a["flags"], a["rec"], a["solid"], a["bm"], a["mm"], None)

    assert mesh(_desc(lattice=0, nz=1)) == _lib.ERR_UNSUPPORTED
    assert mesh(d, flags=4) == _lib.ERR_ARG
    assert mesh(d, brick=0) == _lib.ERR_ARG
    assert mesh(d, bid=255) == _lib.ERR_ARG
    assert mesh(d, solid=p(16385)) == _lib.ERR_ALIGN
    assert mesh(d, rec=p(8196)) == _lib.ERR_ALIGN
    assert mesh(d, pt=None) == _lib.ERR_ARG
    # renderer: missing grid / camera, bad dims, non-positive cells, unaligned buffers
    g = _lib.TriGrid()
    g.cell[:] = [1.0, 1.0, 1.0]
    g.dims[:] = [2, 2, 2]
    g.cell_start = p(1024)
    g.cell_tris = p(2048)
    cam = _lib.Camera()

    def render(grid, camera, pixel=p(4096), depth=p(8192), err=p(16384), h=4, w=4):
        return lib.xlbg_render_mesh(p(32768), 3, p(65536), 1, p(131072), grid, camera, h, w, pixel, depth, None, err,
                                    None)

    assert render(None, ctypes.byref(cam)) == _lib.ERR_ARG
    assert render(ctypes.byref(g), None) == _lib.ERR_ARG
    assert render(ctypes.byref(g), ctypes.byref(cam), h=0) == _lib.ERR_ARG
    assert render(ctypes.byref(g), ctypes.byref(cam), pixel=p(4098)) == _lib.ERR_ALIGN
    assert render(ctypes.byref(g), ctypes.byref(cam), err=None) == _lib.ERR_ARG
    g.dims[:] = [0, 2, 2]
    assert render(ctypes.byref(g), ctypes.byref(cam)) == _lib.ERR_ARG
    g.dims[:] = [2, 2, 2]
    g.cell[:] = [1.0, 0.0, 1.0]
    assert render(ctypes.byref(g), ctypes.byref(cam)) == _lib.ERR_ARG
