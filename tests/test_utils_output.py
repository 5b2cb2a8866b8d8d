"""Field output (xlb/utils/utils.py:50-146): the legacy VTK file and the PNG read back."""

import struct
import zlib

import numpy as np
import pytest

from xlb_gb300.utils import save_fields_vtk, save_image


def _read_vtk(path):
    data = open(path, "rb").read()
    pos = 0
    header = {}
    fields = {}

    def line():
        nonlocal pos
        end = data.index(b"\n", pos)
        text = data[pos:end].decode()
        pos = end + 1
        return text

    assert line().startswith("# vtk DataFile")
    line()
    assert line() == "BINARY"
    assert line() == "DATASET STRUCTURED_POINTS"
    while pos < len(data):
        t = line()
        if not t:
            continue
        key = t.split()[0]
        if key in ("DIMENSIONS", "ORIGIN", "SPACING", "CELL_DATA"):
            header[key] = [float(x) for x in t.split()[1:]]
        elif key == "SCALARS":
            _, name, kind, _ = t.split()
            assert line() == "LOOKUP_TABLE default"
            n = int(header["CELL_DATA"][0])
            dt = ">f4" if kind == "float" else ">f8"
            size = n * np.dtype(dt).itemsize
            fields[name] = np.frombuffer(data[pos:pos + size], dtype=dt)
            pos += size
    return header, fields


@pytest.mark.parametrize("shape", [(4, 3), (3, 4, 5)])
def test_vtk_round_trip(tmp_path, shape):
    rng = np.random.default_rng(1)
    rho = rng.standard_normal(shape).astype(np.float32)
    ux = rng.standard_normal(shape)
    path = save_fields_vtk({"rho": rho, "ux": ux}, 12, output_dir=str(tmp_path), prefix="f")
    assert path.endswith("f_0000012.vtk")
    header, fields = _read_vtk(path)
    dims = [d + 1 for d in shape] + ([1] if len(shape) == 2 else [])
    assert header["DIMENSIONS"] == dims and header["CELL_DATA"] == [np.prod(shape)]
    np.testing.assert_array_equal(fields["rho"].reshape(shape, order="F"), rho)
    np.testing.assert_array_equal(fields["ux"].reshape(shape, order="F"), ux)


def test_vtk_rejects_mismatched_shapes(tmp_path):
    with pytest.raises(AssertionError):
        save_fields_vtk({"a": np.zeros((2, 2)), "b": np.zeros((3, 2))}, 0, output_dir=str(tmp_path))


def test_png_orientation_and_range(tmp_path):
    nx, ny = 5, 3
    fld = np.zeros((nx, ny))
    fld[4, 0] = 2.0  # x = 4, y = 0: bottom-right pixel, maximum
    fld[0, 2] = 1.0  # x = 0, y = 2: top-left pixel
    path = save_image(fld, timestep=7, prefix=str(tmp_path / "img"))
    assert path.endswith("img_0007.png")
    raw = open(path, "rb").read()
    assert raw[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", raw[16:24])
    assert (w, h) == (nx, ny)
    idat_len = struct.unpack(">I", raw[33:37])[0]
    assert raw[37:41] == b"IDAT"
    rows = zlib.decompress(raw[41:41 + idat_len])
    img = np.frombuffer(rows, dtype=np.uint8).reshape(ny, nx + 1)[:, 1:]
    assert img[ny - 1, 4] == 255 and img[0, 0] == 127 and img[1, 1] == 0
    # a (c, nx, ny) field is shown as its magnitude
    vec = np.stack([fld, np.zeros_like(fld)])
    path = save_image(vec, prefix=str(tmp_path / "mag"))
    assert open(path, "rb").read()[:8] == b"\x89PNG\r\n\x1a\n"
