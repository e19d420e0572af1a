"""forge2d_gb300: a GB300-native (sm_103a) implementation of the Box2D v3
world step behind forge2d's backend seam.

The product is the CUDA library ``_build/libforge2d_gb300.so`` with the C ABI
declared in ``include/forge2d_gb300.h``; this package holds its kernels
(``csrc/``), its build recipe, a ctypes binding and a Python mirror of the
forge2d world API.
"""
from .scenes import body_def, revolute_def, shape_def, world_def  # noqa: F401


def build(force: bool = False) -> str:
    from .build import build as _build
    return _build(force=force)


def __getattr__(name):
    if name in ("World", "Body", "Shape", "Joint", "GpuWorld"):
        from . import world as _w
        return getattr(_w, name)
    raise AttributeError(name)
