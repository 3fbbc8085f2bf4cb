"""Known answers of the reference's own shape tests (reference test/test_shape.c:18-100),
restated against the oracle and against the library's host functions (no device)."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from box2c_gb300.capi import Rot, Transform, Vec2
from tests.golden.shapes import Capsule, Circle, _box

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLT_EPS = float(np.finfo(np.float32).eps)
IDENTITY = Transform(Vec2(0.0, 0.0), Rot(1.0, 0.0))


class Segment(C.Structure):
    _fields_ = [("point1", Vec2), ("point2", Vec2)]


class AABB(C.Structure):
    _fields_ = [("lowerBound", Vec2), ("upperBound", Vec2)]


class MassData(C.Structure):
    _fields_ = [("mass", C.c_float), ("center", Vec2), ("rotationalInertia", C.c_float)]


@pytest.fixture(params=["oracle", "library"])
def lib(request, oracle):
    if request.param == "oracle":
        return oracle.lib
    import box2c_gb300
    return C.CDLL(box2c_gb300.build(), mode=os.RTLD_LOCAL | os.RTLD_NOW)


def _fn(lib, name, restype, *argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = list(argtypes)
    return f


def _close(a, b, tol=FLT_EPS):
    return abs(float(np.float32(a)) - float(np.float32(b))) <= tol


def test_shape_aabb_kat(lib):
    # reference test/test_shape.c:75-100
    circle = Circle(Vec2(1.0, 0.0), 1.0)
    b = _fn(lib, "b2ComputeCircleAABB", AABB, C.c_void_p, Transform)(C.addressof(circle), IDENTITY)
    assert _close(b.lowerBound.x, 0.0) and _close(b.lowerBound.y, -1.0)
    assert _close(b.upperBound.x, 2.0) and _close(b.upperBound.y, 1.0)
    box = _box(1.0, 1.0)
    b = _fn(lib, "b2ComputePolygonAABB", AABB, C.c_void_p, Transform)(C.addressof(box), IDENTITY)
    assert _close(b.lowerBound.x, -1.0) and _close(b.lowerBound.y, -1.0)
    assert _close(b.upperBound.x, 1.0) and _close(b.upperBound.y, 1.0)
    segment = Segment(Vec2(0.0, 1.0), Vec2(0.0, -1.0))
    b = _fn(lib, "b2ComputeSegmentAABB", AABB, C.c_void_p, Transform)(C.addressof(segment), IDENTITY)
    assert _close(b.lowerBound.x, 0.0) and _close(b.lowerBound.y, -1.0)
    assert _close(b.upperBound.x, 0.0) and _close(b.upperBound.y, 1.0)


def test_shape_mass_kat(lib):
    # reference test/test_shape.c:18-70 (the capsule against the box that contains it)
    circle = Circle(Vec2(1.0, 0.0), 1.0)
    md = _fn(lib, "b2ComputeCircleMass", MassData, C.c_void_p, C.c_float)(C.addressof(circle), 1.0)
    assert _close(md.mass, math.pi) and md.center.x == 1.0 and md.center.y == 0.0
    assert _close(md.rotationalInertia, 1.5 * np.float32(math.pi))
    poly_mass = _fn(lib, "b2ComputePolygonMass", MassData, C.c_void_p, C.c_float)
    box = _box(1.0, 1.0)
    md = poly_mass(C.addressof(box), 1.0)
    assert _close(md.mass, 4.0) and _close(md.center.x, 0.0) and _close(md.center.y, 0.0)
    assert _close(md.rotationalInertia, np.float32(8.0) / np.float32(3.0), 2 * FLT_EPS)
    capsule = Capsule(Vec2(-1.0, 0.0), Vec2(1.0, 0.0), 1.0)
    mc = _fn(lib, "b2ComputeCapsuleMass", MassData, C.c_void_p, C.c_float)(C.addressof(capsule), 1.0)
    enclosing = _box(1.0 + 1.0, 1.0)  # half-extents radius + half-length, radius (kept alive for the call)
    outer = poly_mass(C.addressof(enclosing), 1.0)
    assert mc.mass < outer.mass and mc.rotationalInertia < outer.rotationalInertia
    assert mc.mass > math.pi  # more than the two end caps' circle
