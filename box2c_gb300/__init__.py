"""box2c_gb300 -- Box2D v3 per-step contact pipeline on one GB300 GPU.

The product is the C shared library ``_build/libbox2d_gb300.so``: it exports the box2d
C API (include/box2d/box2d.h) and runs b2World_Step's broadphase pairs, narrowphase,
graph colouring and soft-step solver with sm_103a kernels.  This module only loads it
(through ctypes, see capi.py) for Python callers, tests and the benchmark.

There is no CPU fallback: if the library is missing or no CUDA device is present,
``load()`` raises.
"""
from __future__ import annotations

import os

from .capi import Backend

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbox2d_gb300.so")
SCENES_PATH = os.path.join(HERE, "_build", "libbox2d_gb300_scenes.so")

_backend: Backend | None = None


def build(verbose: bool = False, force: bool = False) -> str:
    from .compile import build as _build
    return _build(verbose=verbose, force=force)


def load() -> Backend:
    """Loads the GPU library (building it if needed); raises if it cannot run."""
    global _backend
    if _backend is not None:
        return _backend
    if not (os.path.exists(LIB_PATH) and os.path.exists(SCENES_PATH)):
        build()
    b = Backend(LIB_PATH, SCENES_PATH, "gb300")
    import ctypes as C
    b.lib.b2gd_device_ok.restype = C.c_int
    if b.lib.b2gd_device_ok() == 0:
        raise RuntimeError("box2c_gb300: no CUDA device visible; the GB300 library has no CPU fallback")
    _backend = b
    return b


__all__ = ["load", "build", "Backend", "LIB_PATH", "SCENES_PATH"]
