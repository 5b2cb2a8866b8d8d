"""ctypes binding of libxlbg.so (the C ABI declared in include/xlbg.h).

The library is loaded from ``xlb_gb300/lib/libxlbg.so`` (built in-tree by
``xlb_gb300/build.py``).  There is no fallback: if the library is missing or a
call fails, an exception is raised.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libxlbg.so")

ABI_VERSION = 1
MAX_BC = 16
DIAG_SLOTS = 1024
NOALLOC_REC_SCRATCH_BYTES = 4 << 20

OK, ERR_ARG, ERR_UNSUPPORTED, ERR_ALIGN, ERR_CUDA = 0, 1, 2, 3, 4

BC_FULLWAY_BB = 1
BC_HALFWAY_BB = 2
BC_EQUILIBRIUM = 3
BC_ZOUHE_VELOCITY = 4
BC_ZOUHE_PRESSURE = 5
BC_REGULARIZED_VELOCITY = 6
BC_REGULARIZED_PRESSURE = 7
BC_EXTRAPOLATION = 8

BGK, KBC, BGK_PAIR, BGK_SHIFTED, BGK_SHIFTED_SR = 0, 1, 2, 3, 4

KERNEL_AUTO, KERNEL_MARCH, KERNEL_MARCH_WIDE, KERNEL_CELL, KERNEL_TMA_WIDE = 0, 1, 2, 3, 4

MESH_TRI_FLOATS = 39
MESH_EDGE_TESTS = 1


def mesh_solid_bytes(nx, ny, nz):
    """XLBG_MESH_SOLID_BYTES: the padded grid's flags, rounded up to 16 bytes."""
    return ((nx + 2) * (ny + 2) * (nz + 2) + 15) // 16 * 16

EXPORTED = (
    "xlbg_abi_version",
    "xlbg_last_error",
    "xlbg_lattice_tables",
    "xlbg_pack_missing",
    "xlbg_step",
    "xlbg_run",
    "xlbg_step_diag",
    "xlbg_step_diag_noalloc",
    "xlbg_momentum_transfer",
    "xlbg_forward_segment",
    "xlbg_adjoint_segment",
    "xlbg_device_faults",
    "xlbg_debug_force_kernel",
    "xlbg_equilibrium",
    "xlbg_macroscopic",
    "xlbg_indices_mask",
    "xlbg_mesh_mask",
    "xlbg_render_mesh",
)


class XlbgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"xlbg error {code}: {msg}")
        self.code = code


class BCEntry(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int32), ("kind", ctypes.c_int32), ("rho", ctypes.c_double), ("u", ctypes.c_double * 3)]


class Desc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("lattice", ctypes.c_int32),
        ("store", ctypes.c_int32),
        ("compute", ctypes.c_int32),
        ("collision", ctypes.c_int32),
        ("nbc", ctypes.c_int32),
        ("nx", ctypes.c_int64),
        ("ny", ctypes.c_int64),
        ("nz", ctypes.c_int64),
        ("bc", BCEntry * MAX_BC),
    ]


class TriGrid(ctypes.Structure):
    """xlbg_tri_grid: uniform grid of triangle lists for xlbg_render_mesh."""

    _fields_ = [
        ("lo", ctypes.c_float * 3),
        ("cell", ctypes.c_float * 3),
        ("dims", ctypes.c_int32 * 3),
        ("cell_start", ctypes.c_void_p),
        ("cell_tris", ctypes.c_void_p),
    ]


class Camera(ctypes.Structure):
    """xlbg_camera."""

    _fields_ = [
        ("eye", ctypes.c_float * 3),
        ("target", ctypes.c_float * 3),
        ("up", ctypes.c_float * 3),
        ("fov_degrees", ctypes.c_float),
        ("ambient_intensity", ctypes.c_float),
        ("edge_sharpness", ctypes.c_float),
        ("gamma", ctypes.c_float),
    ]


_lock = threading.Lock()
_lib = None

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_DESC = ctypes.POINTER(Desc)

_SIGNATURES = {
    "xlbg_abi_version": ([], ctypes.c_int),
    "xlbg_last_error": ([], ctypes.c_char_p),
    "xlbg_lattice_tables": ([_I32, ctypes.POINTER(_I32), ctypes.POINTER(_D), ctypes.POINTER(_I32)], ctypes.c_int),
    "xlbg_pack_missing": ([_DESC, _P, _P, _P], ctypes.c_int),
    "xlbg_step": ([_DESC, _P, _P, _P, _P, _P, _I64, _P, _D, _I32, _P], ctypes.c_int),
    "xlbg_run": ([_DESC, _P, _P, _P, _P, _P, _I64, _P, _D, _I32, _I32, _P], ctypes.c_int),
    "xlbg_step_diag": ([_DESC, _P, _P, _P, _P, _P, _I64, _P, _D, _I32, _I32, _P, _P, _P], ctypes.c_int),
    "xlbg_step_diag_noalloc": ([_DESC, _P, _P, _P, _P, _P, _I64, _D, _I32, _I32, _P, _P], ctypes.c_int),
    "xlbg_momentum_transfer": ([_DESC, _P, _P, _P, _I32, _P, _P, _P], ctypes.c_int),
    "xlbg_forward_segment": ([_DESC, _P, _I32, _P, _P, _P, _D, _P], ctypes.c_int),
    "xlbg_adjoint_segment": ([_DESC, _P, _I32, _P, _P, _P, _P, _I64, _P, _P, _P, _D, _P], ctypes.c_int),
    "xlbg_device_faults": ([_I32], ctypes.c_int),
    "xlbg_debug_force_kernel": ([_I32], ctypes.c_int),
    "xlbg_equilibrium": ([_DESC, _P, _P, _D, ctypes.POINTER(_D), _P, _P], ctypes.c_int),
    "xlbg_macroscopic": ([_DESC, _P, _P, _P, _P], ctypes.c_int),
    "xlbg_indices_mask": ([_DESC, _P, _I64, _I32, _I32, _P, _P, _P], ctypes.c_int),
    "xlbg_render_mesh": ([_P, _I64, _P, _I64, _P, ctypes.POINTER(TriGrid), ctypes.POINTER(Camera), _I32, _I32,
                          _P, _P, _P, _P, _P], ctypes.c_int),
    "xlbg_mesh_mask": ([_DESC, _P, _I64, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
}


def load(build_if_missing=True):
    """Load libxlbg.so (building it first when absent and nvcc is available)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH) and build_if_missing:
            from xlb_gb300 import build as _build

            _build.build()
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libxlbg.so not found at {LIB_PATH}; run xlb_gb300/build.py")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        if lib.xlbg_abi_version() != ABI_VERSION:
            raise ImportError("libxlbg.so ABI version mismatch; rebuild it")
        _lib = lib
        return lib


def check(status):
    if status != OK:
        msg = load().xlbg_last_error().decode(errors="replace")
        raise XlbgError(status, msg)


def lattice_tables(lattice):
    """(c (q, d), w (q,), opp (q,)) as compiled into the kernels."""
    import numpy as np

    c = (_I32 * (27 * 3))()
    w = (_D * 27)()
    o = (_I32 * 27)()
    q = load().xlbg_lattice_tables(lattice, c, w, o)
    if q < 0:
        check(-q)
    d = 2 if lattice == 0 else 3
    return (
        np.array(c[: q * d], dtype=np.int64).reshape(q, d),
        np.array(w[:q], dtype=np.float64),
        np.array(o[:q], dtype=np.int64),
    )


def ptr(t):
    """Device pointer of a torch tensor, or None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def mark_written(*tensors):
    """Bump the version counter of tensors a C-ABI call wrote in place.

    Writes through raw pointers are invisible to torch; caches keyed on a
    tensor's ``_version`` (the stepper's packed missing bits) see the change
    only through this."""
    import torch

    for t in tensors:
        if t is not None:
            torch.autograd.graph.increment_version(t)


class forced_kernel:
    """Context manager: run the step entry points on one kernel variant
    (KERNEL_*) inside the block, back to the automatic choice after it."""

    def __init__(self, kernel):
        self.kernel = kernel

    def __enter__(self):
        check(load().xlbg_debug_force_kernel(self.kernel))
        return self

    def __exit__(self, *exc):
        check(load().xlbg_debug_force_kernel(KERNEL_AUTO))


def stream_handle(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _raw_stream_getter():
    import torch

    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return raw
    return lambda device: torch.cuda.current_stream(device).cuda_stream


_raw_stream = None


def raw_stream(device_index):
    """cudaStream_t (as an int) of torch's current stream on a device: the
    per-step calls' cheap form of stream_handle (0.1 us against 3 us)."""
    global _raw_stream
    if _raw_stream is None:
        _raw_stream = _raw_stream_getter()
    return _raw_stream(device_index)
