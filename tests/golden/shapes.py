"""Seeded random shape pairs for manifold golden vectors (shared by the generator and
the tests so both sides rebuild the same inputs from the seed)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from box2c_gb300.capi import Vec2, Rot, Transform


class Polygon(C.Structure):
    _fields_ = [("vertices", Vec2 * 8), ("normals", Vec2 * 8), ("centroid", Vec2), ("radius", C.c_float),
                ("count", C.c_int32)]


class Circle(C.Structure):
    _fields_ = [("center", Vec2), ("radius", C.c_float)]


class Capsule(C.Structure):
    _fields_ = [("center1", Vec2), ("center2", Vec2), ("radius", C.c_float)]


class ManifoldPoint(C.Structure):
    _fields_ = [("point", Vec2), ("anchorA", Vec2), ("anchorB", Vec2), ("separation", C.c_float),
                ("normalImpulse", C.c_float), ("tangentImpulse", C.c_float), ("maxNormalImpulse", C.c_float),
                ("normalVelocity", C.c_float), ("id", C.c_uint16), ("persisted", C.c_bool)]


class Manifold(C.Structure):
    _fields_ = [("points", ManifoldPoint * 2), ("normal", Vec2), ("pointCount", C.c_int32)]


def _box(hx, hy, radius=0.0):
    p = Polygon()
    vs = [(-hx, -hy), (hx, -hy), (hx, hy), (-hx, hy)]
    ns = [(0, -1), (1, 0), (0, 1), (-1, 0)]
    for i in range(4):
        p.vertices[i] = Vec2(*vs[i])
        p.normals[i] = Vec2(*ns[i])
    p.count = 4
    p.radius = radius
    return p


def _ngon(n, r):
    # vertices and normals are rounded to float32 once; the same bits reach both sides
    p = Polygon()
    pts = [(r * math.cos(2 * math.pi * k / n), r * math.sin(2 * math.pi * k / n)) for k in range(n)]
    pts = [(float(np.float32(x)), float(np.float32(y))) for x, y in pts]
    for i in range(n):
        x1, y1 = pts[i]
        x2, y2 = pts[(i + 1) % n]
        ex, ey = x2 - x1, y2 - y1
        l = math.hypot(ex, ey)
        p.vertices[i] = Vec2(x1, y1)
        p.normals[i] = Vec2(float(np.float32(ey / l)), float(np.float32(-ex / l)))
    p.count = n
    return p


def _xf(rng, spread):
    a = rng.uniform(-math.pi, math.pi)
    return Transform(Vec2(rng.uniform(-spread, spread), rng.uniform(-spread, spread)),
                     Rot(float(np.float32(math.cos(a))), float(np.float32(math.sin(a)))))


def random_pairs(seed: int, count: int):
    """List of (function name, shapeA, xfA, shapeB, xfB)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        kind = k % 5
        xa = _xf(rng, 0.3)
        xb = _xf(rng, 1.4)
        if kind == 0:
            a = _box(rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
            b = _box(rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.choice([0.0, 0.05]))
            out.append(("b2CollidePolygons", a, xa, b, xb))
        elif kind == 1:
            a = _ngon(int(rng.integers(3, 9)), rng.uniform(0.3, 0.9))
            b = _ngon(int(rng.integers(3, 9)), rng.uniform(0.3, 0.9))
            out.append(("b2CollidePolygons", a, xa, b, xb))
        elif kind == 2:
            a = _box(rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
            b = Circle(Vec2(0.0, 0.0), rng.uniform(0.1, 0.6))
            out.append(("b2CollidePolygonAndCircle", a, xa, b, xb))
        elif kind == 3:
            a = Circle(Vec2(0.0, 0.0), rng.uniform(0.1, 0.6))
            b = Circle(Vec2(0.0, 0.0), rng.uniform(0.1, 0.6))
            out.append(("b2CollideCircles", a, xa, b, xb))
        else:
            a = Capsule(Vec2(-0.5, 0.0), Vec2(0.5, 0.0), rng.uniform(0.05, 0.3))
            b = Capsule(Vec2(0.0, -0.4), Vec2(0.0, 0.4), rng.uniform(0.05, 0.3))
            out.append(("b2CollideCapsules", a, xa, b, xb))
    return out


class Segment(C.Structure):
    _fields_ = [("point1", Vec2), ("point2", Vec2)]


class SmoothSegment(C.Structure):
    _fields_ = [("ghost1", Vec2), ("segment", Segment), ("ghost2", Vec2), ("chainId", C.c_int32)]


class DistanceCache(C.Structure):
    _fields_ = [("count", C.c_uint16), ("indexA", C.c_uint8 * 3), ("indexB", C.c_uint8 * 3)]


def _f32(x):
    return float(np.float32(x))


def random_smooth_pairs(seed: int, count: int):
    """Chain links (a segment with ghost vertices bent convex or concave at either end)
    against circles, capsules, boxes and n-gons placed around the link's collision side.
    List of (function name, smooth segment, xfA, shapeB, xfB)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        half = rng.uniform(0.4, 1.2)
        s = SmoothSegment()
        s.segment.point1 = Vec2(_f32(half), 0.0)
        s.segment.point2 = Vec2(_f32(-half), 0.0)  # right to left: the upper side collides
        b1, b2 = rng.uniform(-0.8, 0.8, size=2)
        s.ghost1 = Vec2(_f32(half + 1.0), _f32(b1))
        s.ghost2 = Vec2(_f32(-half - 1.0), _f32(b2))
        s.chainId = -1
        xa = _xf(rng, 0.2)
        a = rng.uniform(-math.pi, math.pi)
        # B's centre in A's frame: mostly above the link (its collision side), some behind
        lx, ly = rng.uniform(-1.8, 1.8), rng.uniform(-0.3, 0.9)
        c, sn = xa.q.c, xa.q.s
        xb = Transform(Vec2(_f32(xa.p.x + c * lx - sn * ly), _f32(xa.p.y + sn * lx + c * ly)),
                       Rot(_f32(math.cos(a)), _f32(math.sin(a))))
        kind = k % 4
        if kind == 0:
            out.append(("b2CollideSmoothSegmentAndCircle", s, xa, Circle(Vec2(0.0, 0.0), rng.uniform(0.1, 0.6)), xb))
        elif kind == 1:
            b = Capsule(Vec2(-0.4, 0.0), Vec2(0.4, 0.0), rng.uniform(0.05, 0.3))
            out.append(("b2CollideSmoothSegmentAndCapsule", s, xa, b, xb))
        elif kind == 2:
            b = _box(rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.choice([0.0, 0.05]))
            out.append(("b2CollideSmoothSegmentAndPolygon", s, xa, b, xb))
        else:
            b = _ngon(int(rng.integers(3, 9)), rng.uniform(0.3, 0.9))
            out.append(("b2CollideSmoothSegmentAndPolygon", s, xa, b, xb))
    return out


def collide_smooth(lib, entry) -> np.ndarray:
    """Calls a smooth segment manifold function twice, from an empty closest-feature cache
    and again from the cache the first call left; returns both manifolds and caches."""
    name, s, xa, b, xb = entry
    fn = getattr(lib, name)
    fn.restype = Manifold
    cache = DistanceCache()
    outs = []
    for _ in range(2):
        if name.endswith("Circle"):
            fn.argtypes = [C.c_void_p, Transform, C.c_void_p, Transform]
            m = fn(C.addressof(s), xa, C.addressof(b), xb)
        else:
            fn.argtypes = [C.c_void_p, Transform, C.c_void_p, Transform, C.c_void_p]
            m = fn(C.addressof(s), xa, C.addressof(b), xb, C.addressof(cache))
        c = [float(cache.count)] + [float(v) for v in cache.indexA] + [float(v) for v in cache.indexB]
        outs.append(np.concatenate([manifold_array(m), np.array(c, np.float32)]))
    return np.concatenate(outs)


def manifold_array(m: Manifold) -> np.ndarray:
    """Flattens a manifold into 2 + 1 + 2*8 float32 words (ids bit-cast)."""
    vals = [m.normal.x, m.normal.y, float(m.pointCount)]
    for i in range(2):
        p = m.points[i]
        vals += [p.point.x, p.point.y, p.anchorA.x, p.anchorA.y, p.anchorB.x, p.anchorB.y, p.separation, float(p.id)]
    return np.array(vals, np.float32)


__all__ = ["Polygon", "Circle", "Capsule", "Manifold", "Transform", "SmoothSegment", "DistanceCache", "random_pairs",
           "random_smooth_pairs", "collide_smooth", "manifold_array"]
