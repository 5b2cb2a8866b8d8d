"""Make ``import xlb`` work from the XLB source tree without jax/warp installed.

Test infrastructure only.  ``install()`` puts the Warp emulator (refshim/warp)
on sys.path and registers stand-in modules for packages XLB imports at module
scope but that the Warp stepper path never calls: jax (its ``jit`` is the
identity, so JAX method bodies stay plain functions), matplotlib, pyvista,
trimesh, cupy.
"""

import importlib.abc
import importlib.machinery
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
STUBBED = ("jax", "matplotlib", "pyvista", "trimesh", "cupy", "kvikio", "mpi4py", "pxr", "nvtx")


class _Anything:
    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __getitem__(self, k):
        return _Anything()

    def __iter__(self):
        return iter(())


def _jit(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything()


class _Finder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path=None, target=None):
        if name.split(".")[0] in STUBBED:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = _StubModule(spec.name)
        m.__path__ = []
        if spec.name == "jax":
            m.jit = _jit
            m.vmap = lambda f, *a, **k: f
            m.config = types.SimpleNamespace(update=lambda *a, **k: None)
            m.devices = lambda *a, **k: [types.SimpleNamespace(platform="cpu")]
            m.device_count = lambda: 1
        return m

    def exec_module(self, module):
        return None


def install(reference_root):
    if HERE not in sys.path:
        sys.path.insert(0, HERE)
    if not any(isinstance(f, _Finder) for f in sys.meta_path):
        sys.meta_path.insert(0, _Finder())
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
