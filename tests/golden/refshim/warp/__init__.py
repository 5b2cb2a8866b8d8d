"""A minimal CPU emulation of the NVIDIA Warp Python API, enough to execute XLB's
Warp stepper source unmodified for golden-vector generation.

Test infrastructure only (used by tests/golden/make_golden.py in the container
that holds the XLB source tree).  Semantics modelled:

* ``wp.vec`` / ``wp.mat`` value types with element dtype (numpy scalars, so FP64
  arithmetic is IEEE double, op by op, no fusion);
* ``@wp.func`` passes vectors by value (arguments are copied on entry);
* ``@wp.kernel`` + ``wp.launch`` run the kernel body once per thread index, in
  row-major order, sequentially;
* ``wp.static``, ``wp.constant`` are identities;
* builtins used by XLB's stepper path: dot, cw_div, abs, sqrt, atomic_add, tid;
* for the mesh boundary masker: ``mat33`` values (from 9 scalars row by row, a
  scalar fill, or 3 vectors as columns), ``transpose``, ``cross``, ``normalize``,
  ``length``, and ``Mesh`` with ``mesh_query_aabb`` (faces whose bounds meet the
  query box, closed intervals), ``mesh_eval_position`` (u*p0 + v*p1 +
  (1-u-v)*p2) and ``mesh_eval_face_normal`` (normalize(cross(p1-p0, p2-p0))).
  ``m[i]`` of a matrix is a copy of row i, so ``m[i][j] = x`` leaves ``m``
  unchanged, as in Warp's generated code for a local matrix;
  ``NESTED_STORES_WRITE = True`` makes it write into ``m`` instead.

Python-scope builtin calls on Python floats (``wp.sqrt(3.0)``) evaluate in
float32, the way Warp types bare Python floats.  Kernel scalar arguments keep
their Python type (Warp would type a bare float as float32; this emulator does
not model that).
"""

import itertools

import numpy as np

float16 = np.float16
float32 = np.float32
float64 = np.float64
int8 = np.int8
int32 = np.int32
int64 = np.int64
uint8 = np.uint8
uint32 = np.uint32
uint64 = np.uint64
bool = np.bool_  # noqa: A001  (Warp's name)

_vec_types = {}


class _Vec:
    __array_ufunc__ = None  # make numpy scalars defer to our reflected operators
    length = 0
    dtype = float32

    def __init__(self, *args):
        n, dt = self.length, self.dtype
        if not args:
            vals = [dt(0)] * n
        elif len(args) == 1 and hasattr(args[0], "__len__") and not isinstance(args[0], str):
            vals = [dt(v) for v in args[0]]
        elif len(args) == 1 and n > 1:  # a scalar fills every component
            vals = [dt(args[0])] * n
        else:
            vals = [dt(v) for v in args]
        if len(vals) != n:
            raise ValueError(f"vector of length {n} built from {len(vals)} values")
        self.v = vals

    def copy(self):
        c = type(self).__new__(type(self))
        c.v = list(self.v)
        return c

    def __len__(self):
        return self.length

    def __iter__(self):
        return iter(self.v)

    def __getitem__(self, i):
        return self.v[int(i)]

    def __setitem__(self, i, x):
        self.v[int(i)] = self.dtype(x)
        owner = getattr(self, "_owner", None)
        if owner is not None:
            owner[0].a[owner[1], int(i)] = x

    def _map(self, fn):
        c = type(self).__new__(type(self))
        c.v = [self.dtype(fn(a)) for a in self.v]
        return c

    def _zip(self, other, fn):
        c = type(self).__new__(type(self))
        c.v = [self.dtype(fn(a, b)) for a, b in zip(self.v, other.v)]
        return c

    def __add__(self, o):
        return self._zip(o, lambda a, b: a + b) if isinstance(o, _Vec) else self._map(lambda a: a + o)

    def __sub__(self, o):
        return self._zip(o, lambda a, b: a - b) if isinstance(o, _Vec) else self._map(lambda a: a - o)

    def __mul__(self, o):
        if isinstance(o, _Vec):
            raise TypeError("vec * vec is not defined; use wp.cw_mul")
        return self._map(lambda a: a * o)

    def __rmul__(self, o):
        return self._map(lambda a: o * a)

    def __truediv__(self, o):
        return self._map(lambda a: a / o)

    def __neg__(self):
        return self._map(lambda a: -a)

    def __repr__(self):
        return f"vec{self.length}({', '.join(map(str, self.v))})"


def _vec_type(length, dtype):
    key = (int(length), dtype)
    if key not in _vec_types:
        _vec_types[key] = type(f"vec{length}_{getattr(dtype, '__name__', dtype)}", (_Vec,), {"length": int(length), "dtype": dtype})
    return _vec_types[key]


def vec(*args, length=None, dtype=None):
    """``wp.vec(length, dtype)`` is a type; ``wp.vec(value, length=n)`` a value."""
    if length is None:
        return _vec_type(args[0], dtype)
    if not args:
        return _vec_type(length, dtype)
    dt = dtype or (type(args[0]) if isinstance(args[0], np.generic) else float32)
    return _vec_type(length, dt)(*args)


vec2i = _vec_type(2, int32)
vec3i = _vec_type(3, int32)
vec2f = _vec_type(2, float32)
vec3f = _vec_type(3, float32)
vec2d = _vec_type(2, float64)
vec3d = _vec_type(3, float64)
vec3 = vec3f
vec2 = vec2f


NESTED_STORES_WRITE = False


class _Mat:
    __array_ufunc__ = None

    def __init__(self, a, dtype):
        self.a = np.asarray(a).astype(dtype)
        self.dtype = dtype

    def __getitem__(self, idx):
        if isinstance(idx, tuple):
            return self.a[tuple(int(i) for i in idx)]
        row = _vec_type(self.a.shape[1], self.dtype)(self.a[int(idx)])
        if NESTED_STORES_WRITE:
            row._owner = (self, int(idx))  # element stores write through (see _Vec.__setitem__)
        return row

    def __setitem__(self, idx, x):
        if isinstance(idx, tuple):
            self.a[tuple(int(i) for i in idx)] = x
        else:
            self.a[int(idx)] = np.asarray(list(x), dtype=self.dtype)


def mat(shape, dtype=float32):
    def make(a):
        m = _Mat(a, dtype)
        if m.a.shape != tuple(shape):
            raise ValueError(f"matrix data of shape {m.a.shape}, type is {tuple(shape)}")
        return m

    return make


def _mat33_ctor(dtype):
    def make(*args):
        if len(args) == 1 and not isinstance(args[0], _Vec):
            return _Mat(np.full((3, 3), args[0]), dtype)
        if len(args) == 3 and all(isinstance(a, _Vec) for a in args):
            return _Mat(np.array([list(a.v) for a in args]).T, dtype)  # vectors are columns
        if len(args) == 9:
            return _Mat(np.array(args).reshape(3, 3), dtype)
        raise ValueError(f"mat33 from {len(args)} arguments")

    return make


mat33f = mat33 = _mat33_ctor(float32)
mat33d = _mat33_ctor(float64)


def mat44(*args):
    """16 scalars, row by row."""
    if len(args) != 16:
        raise ValueError(f"mat44 from {len(args)} arguments")
    return _Mat(np.array([float32(a) for a in args]).reshape(4, 4), float32)


def transpose(m):
    return _Mat(m.a.T.copy(), m.dtype)


# ----------------------------------------------------------------------------- arrays


class _Array(np.ndarray):
    """numpy array with Warp's ``.numpy()``."""

    def numpy(self):
        return np.asarray(self)


class _VecArray:
    """1-D array whose elements are vectors (``wp.zeros(n, dtype=vec_type)``)."""

    def __init__(self, n, vt):
        self.data = [vt() for _ in range(n)]
        self.shape = (n,)

    def __getitem__(self, i):
        return self.data[int(i)]

    def __setitem__(self, i, x):
        self.data[int(i)] = x

    def numpy(self):
        return np.array([v.v for v in self.data])


def _as_array(a, dtype=None):
    if isinstance(dtype, type) and issubclass(dtype, _Vec):
        dtype = dtype.dtype  # array of vectors: trailing axis of the vector's length
    arr = np.asarray(a) if dtype is None else np.asarray(a).astype(dtype)
    return np.ascontiguousarray(arr).view(_Array)


def array(data=None, dtype=None, shape=None, device=None, **kw):
    """``wp.array(data, dtype)`` copies ``data``; ``wp.array(dtype=...)`` alone is an annotation."""
    if data is None:
        return None
    return _as_array(data, dtype)


def _annotation(*a, **k):
    return None


array1d = array2d = array3d = array4d = _annotation


def zeros(shape, dtype=float32, device=None, **kw):
    if isinstance(dtype, type) and issubclass(dtype, _Vec):
        n = shape if isinstance(shape, int) else int(np.prod(shape))
        return _VecArray(n, dtype)
    return np.zeros(shape, dtype=dtype).view(_Array)


def full(shape, value, dtype=float32, device=None, **kw):
    return np.full(shape, value, dtype=dtype).view(_Array)


def copy(dest, src, *a, **k):
    dest[...] = src


def from_numpy(a, dtype=None, **kw):
    return _as_array(a, dtype)


# ----------------------------------------------------------------------------- functions and kernels


def func(f):
    def call(*args, **kwargs):
        args = [a.copy() if isinstance(a, _Vec) else a for a in args]
        return f(*args, **kwargs)

    call.__wrapped__ = f
    call.__name__ = getattr(f, "__name__", "func")
    return call


class _Kernel:
    """A kernel object (not a function, so a kernel defined in a class body is
    not bound to instances, as with Warp's Kernel)."""

    def __init__(self, f):
        self.f = f
        self.__name__ = getattr(f, "__name__", "kernel")

    def __call__(self, *args):
        return self.f(*args)


def kernel(f=None, **kw):
    if f is None:
        return lambda g: _Kernel(g)
    return _Kernel(f)


_current_tid = None


def tid():
    return _current_tid


def launch(kernel, dim, inputs=(), outputs=(), device=None, **kw):
    global _current_tid
    args = list(inputs) + list(outputs)
    if isinstance(dim, (int, np.integer)):
        it = ((i,) for i in range(int(dim)))
        single = True
    else:
        it = itertools.product(*[range(int(d)) for d in dim])
        single = False
    try:
        for t in it:
            _current_tid = t[0] if single else tuple(int32(v) for v in t)
            kernel(*args)
    finally:
        _current_tid = None


def static(x):
    return x


def constant(x):
    return x


def init():
    return None


def synchronize():
    return None


# ----------------------------------------------------------------------------- builtins


def dot(a, b):
    s = a.dtype(0)
    for x, y in zip(a.v, b.v):
        s = s + x * y
    return s


def cw_div(a, b):
    return a._zip(b, lambda x, y: x / y)


def cw_mul(a, b):
    return a._zip(b, lambda x, y: x * y)


def abs(x):  # noqa: A001
    return np.abs(x)


def sqrt(x):
    if isinstance(x, float):  # Python-scope call on a bare float: float32 in Warp
        return float(np.sqrt(np.float32(x)))
    return np.sqrt(x)


def max(a, b):  # noqa: A001
    return a if a >= b else b


def min(a, b):  # noqa: A001
    return a if a <= b else b


def length(v):
    return np.sqrt(dot(v, v))


def cross(a, b):
    return type(a)(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def normalize(a):
    n = length(a)
    return a / n if n > 0 else type(a)()


_meshes = {}


class Mesh:
    """Triangle mesh: points (N, 3), indices (3T,).  ``id`` keys the registry;
    ``mesh_get(id)`` returns the mesh itself (its ``points`` and flat ``indices``)."""

    def __init__(self, points, indices, **kw):
        self.points = np.asarray(points, dtype=float32)
        self.indices = np.asarray(indices).astype(np.int64).reshape(-1)
        self.tri_index = self.indices.reshape(-1, 3)
        tri = self.points[self.tri_index]  # (T, 3, 3)
        self.lowers = tri.min(axis=1)
        self.uppers = tri.max(axis=1)
        self.id = uint64(len(_meshes) + 1)
        _meshes[int(self.id)] = self


def mesh_query_aabb(mesh_id, lower, upper):
    m = _meshes[int(mesh_id)]
    lo = np.array(lower.v, dtype=float32)
    hi = np.array(upper.v, dtype=float32)
    hit = np.all((m.lowers <= hi) & (m.uppers >= lo), axis=1)
    return iter(int(f) for f in np.nonzero(hit)[0])


def _mesh_vertex(m, f, k):
    return vec3f(m.points[m.tri_index[f, k]])


def mesh_get(mesh_id):
    return _meshes[int(mesh_id)]


class _RayQuery:
    def __init__(self, result, t=0.0, u=0.0, v=0.0, sign=1.0, normal=None, face=-1):
        self.result = result
        self.t, self.u, self.v, self.sign, self.face = float32(t), float32(u), float32(v), float32(sign), int32(face)
        self.normal = normal if normal is not None else vec3f()


def _woop(org, d, p, q, r):
    """Watertight ray-triangle test (Woop, Benthin, Wald, JCGT 2013) in float32,
    without its double-precision fallback: (hit, t, u, v), u weighting p, v q."""
    ad = [abs(d[0]), abs(d[1]), abs(d[2])]
    kz = 0
    if ad[1] > ad[kz]:
        kz = 1
    if ad[2] > ad[kz]:
        kz = 2
    kx = (kz + 1) % 3
    ky = (kx + 1) % 3
    if d[kz] < 0:
        kx, ky = ky, kx
    sx = d[kx] / d[kz]
    sy = d[ky] / d[kz]
    sz = float32(1) / d[kz]
    a, b, c = p - org, q - org, r - org
    ax = a[kx] - sx * a[kz]
    ay = a[ky] - sy * a[kz]
    bx = b[kx] - sx * b[kz]
    by = b[ky] - sy * b[kz]
    cx = c[kx] - sx * c[kz]
    cy = c[ky] - sy * c[kz]
    U = cx * by - cy * bx
    V = ax * cy - ay * cx
    W = bx * ay - by * ax
    if (U < 0 or V < 0 or W < 0) and (U > 0 or V > 0 or W > 0):
        return False, 0, 0, 0
    det = (U + V) + W
    if det == 0:
        return False, 0, 0, 0
    T = (U * (sz * a[kz]) + V * (sz * b[kz])) + W * (sz * c[kz])
    rcp = float32(1) / det
    t = T * rcp
    if not t >= 0:
        return False, 0, 0, 0
    return True, t, U * rcp, V * rcp


def mesh_query_ray(mesh_id, start, direction, max_t):
    """Closest hit with t < max_t over all faces; equal t keeps the lower face."""
    m = _meshes[int(mesh_id)]
    org = vec3f(start)
    d = vec3f(direction)
    best = None
    min_t = float32(max_t)
    for f in range(m.tri_index.shape[0]):
        p, q, r = (_mesh_vertex(m, f, k) for k in range(3))
        hit, t, u, v = _woop(org, d, p, q, r)
        if hit and t < min_t:
            min_t = t
            best = (t, u, v, f, normalize(cross(q - p, r - p)))
    if best is None:
        return _RayQuery(False)
    t, u, v, f, n = best
    return _RayQuery(True, t, u, v, 1.0, n, f)


def pow(x, y):  # noqa: A001
    return float32(np.power(float32(x), float32(y)))


def clamp(x, lo, hi):
    return lo if x < lo else (hi if x > hi else x)


def mesh_eval_position(mesh_id, face, u, v):
    m = _meshes[int(mesh_id)]
    p, q, r = (_mesh_vertex(m, face, k) for k in range(3))
    u, v = float32(u), float32(v)
    return p * u + q * v + r * (float32(1) - u - v)


def mesh_eval_face_normal(mesh_id, face):
    m = _meshes[int(mesh_id)]
    p, q, r = (_mesh_vertex(m, face, k) for k in range(3))
    return normalize(cross(q - p, r - p))


def atomic_add(arr, i, value):
    arr[i] = arr[i] + value
    return arr[i]


class _Permissive:
    """Stand-in for Warp names the stepper path never calls (import-time only)."""

    def __call__(self, *a, **k):
        return self

    def __getattr__(self, name):
        return self


def __getattr__(name):
    return _Permissive()
