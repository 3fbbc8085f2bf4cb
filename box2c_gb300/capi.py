"""ctypes mirror of the box2d C API (include/box2d/*.h) and of the scene generators.

The same bindings drive any shared object that exports the box2d C API: this
package's GPU library, and (in tests only) the plain-C oracle and the reference
build.  Struct layouts follow include/box2d/{math_functions,id,types,inspect}.h, which
in turn keep the layouts of the reference include/box2d headers.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np


class Vec2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class Rot(C.Structure):
    _fields_ = [("c", C.c_float), ("s", C.c_float)]


class Transform(C.Structure):
    _fields_ = [("p", Vec2), ("q", Rot)]


class WorldId(C.Structure):
    _fields_ = [("index1", C.c_uint16), ("revision", C.c_uint16)]


class BodyId(C.Structure):
    _fields_ = [("index1", C.c_int32), ("world0", C.c_uint16), ("revision", C.c_uint16)]


ShapeId = BodyId
JointId = BodyId


class ShapePairEvent(C.Structure):
    """b2ContactBeginTouchEvent / b2ContactEndTouchEvent / b2Sensor*TouchEvent layout."""
    _fields_ = [("shapeIdA", BodyId), ("shapeIdB", BodyId)]


class ContactHitEvent(C.Structure):
    _fields_ = [("shapeIdA", BodyId), ("shapeIdB", BodyId), ("point", Vec2), ("normal", Vec2), ("approachSpeed", C.c_float)]


class ContactEvents(C.Structure):
    _fields_ = [("beginEvents", C.POINTER(ShapePairEvent)), ("endEvents", C.POINTER(ShapePairEvent)),
                ("hitEvents", C.POINTER(ContactHitEvent)), ("beginCount", C.c_int32), ("endCount", C.c_int32),
                ("hitCount", C.c_int32)]


class SensorEvents(C.Structure):
    _fields_ = [("beginEvents", C.POINTER(ShapePairEvent)), ("endEvents", C.POINTER(ShapePairEvent)),
                ("beginCount", C.c_int32), ("endCount", C.c_int32)]


class Counters(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "staticBodyCount", "bodyCount", "shapeCount", "contactCount", "jointCount",
        "islandCount", "stackUsed", "staticTreeHeight", "treeHeight", "byteCount",
        "taskCount")] + [("colorCounts", C.c_int32 * 12)]


class Profile(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "step", "pairs", "collide", "solve", "buildIslands", "solveConstraints",
        "prepareTasks", "solverTasks", "prepareConstraints", "integrateVelocities",
        "warmStart", "solveVelocities", "integratePositions", "relaxVelocities",
        "applyRestitution", "storeImpulses", "finalizeBodies", "splitIslands",
        "sleepIslands", "hitEvents", "broadphase", "continuous")]


class InspectPoint(C.Structure):
    _fields_ = [("anchorA", C.c_float * 2), ("anchorB", C.c_float * 2), ("point", C.c_float * 2),
                ("separation", C.c_float), ("normalImpulse", C.c_float),
                ("tangentImpulse", C.c_float), ("maxNormalImpulse", C.c_float),
                ("normalVelocity", C.c_float), ("id", C.c_int32), ("persisted", C.c_int32)]


class InspectContact(C.Structure):
    _fields_ = [("contactId", C.c_int32), ("shapeIdA", C.c_int32), ("shapeIdB", C.c_int32),
                ("colorIndex", C.c_int32), ("localIndex", C.c_int32), ("touching", C.c_int32),
                ("pointCount", C.c_int32), ("normal", C.c_float * 2), ("friction", C.c_float),
                ("restitution", C.c_float), ("points", InspectPoint * 2)]


class InspectShape(C.Structure):
    _fields_ = [("aabb", C.c_float * 4), ("fatAABB", C.c_float * 4), ("proxyKey", C.c_int32),
                ("bodyId", C.c_int32)]


BODY_FLOATS = 8


def _load(path: str) -> C.CDLL:
    # RTLD_LOCAL keeps each backend's b2* symbols private, so several backends can
    # live in one process without interposing on one another.
    return C.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)


class Backend:
    """One implementation of the box2d C API plus its scene generator library."""

    def __init__(self, lib_path: str, scenes_path: str, name: str):
        self.name = name
        self.lib = _load(lib_path)
        self.scenes = _load(scenes_path)
        L, S = self.lib, self.scenes
        L.b2World_Step.argtypes = [WorldId, C.c_float, C.c_int]
        L.b2World_Step.restype = None
        L.b2DestroyWorld.argtypes = [WorldId]
        L.b2DestroyWorld.restype = None
        L.b2World_GetCounters.argtypes = [WorldId]
        L.b2World_GetCounters.restype = Counters
        L.b2World_GetProfile.argtypes = [WorldId]
        L.b2World_GetProfile.restype = Profile
        L.b2World_InspectBodies.argtypes = [WorldId, C.c_void_p, C.c_int]
        L.b2World_InspectBodies.restype = C.c_int
        L.b2World_InspectShapes.argtypes = [WorldId, C.c_void_p, C.c_int]
        L.b2World_InspectShapes.restype = C.c_int
        L.b2World_InspectContacts.argtypes = [WorldId, C.c_void_p, C.c_int]
        L.b2World_InspectContacts.restype = C.c_int
        L.b2World_InspectIslands.argtypes = [WorldId, C.c_void_p, C.c_int]
        L.b2World_InspectIslands.restype = C.c_int
        L.b2Body_GetPosition.argtypes = [BodyId]
        L.b2Body_GetPosition.restype = Vec2
        L.b2Body_GetRotation.argtypes = [BodyId]
        L.b2Body_GetRotation.restype = Rot
        L.b2Body_GetLinearVelocity.argtypes = [BodyId]
        L.b2Body_GetLinearVelocity.restype = Vec2
        L.b2Body_GetAngularVelocity.argtypes = [BodyId]
        L.b2Body_GetAngularVelocity.restype = C.c_float
        L.b2Body_SetLinearVelocity.argtypes = [BodyId, Vec2]
        L.b2Body_SetLinearVelocity.restype = None
        for name, idt in (("b2DestroyBody", BodyId), ("b2DestroyShape", ShapeId), ("b2DestroyJoint", JointId)):
            getattr(L, name).argtypes = [idt]
            getattr(L, name).restype = None
        for name, idt in (("b2Body_IsValid", BodyId), ("b2Shape_IsValid", ShapeId), ("b2Joint_IsValid", JointId)):
            getattr(L, name).argtypes = [idt]
            getattr(L, name).restype = C.c_bool
        L.b2World_GetContactEvents.argtypes = [WorldId]
        L.b2World_GetContactEvents.restype = ContactEvents
        L.b2World_GetSensorEvents.argtypes = [WorldId]
        L.b2World_GetSensorEvents.restype = SensorEvents
        L.b2Body_GetShapes.argtypes = [BodyId, C.c_void_p, C.c_int]
        L.b2Body_GetShapes.restype = C.c_int
        S.b2s_pyramid.argtypes = [C.c_int, C.c_float, C.c_uint64]
        S.b2s_pyramid.restype = WorldId
        S.b2s_tumbler.argtypes = [C.c_int, C.c_uint64, C.c_int]
        S.b2s_tumbler.restype = WorldId
        S.b2s_drop_boxes.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float]
        S.b2s_drop_boxes.restype = WorldId
        S.b2s_drop_shapes.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        S.b2s_drop_shapes.restype = WorldId
        S.b2s_hello_world.argtypes = [C.POINTER(BodyId)]
        S.b2s_hello_world.restype = WorldId
        S.b2s_tilted_stacks.argtypes = []
        S.b2s_tilted_stacks.restype = WorldId
        S.b2s_joint_grid.argtypes = [C.c_int, C.c_float]
        S.b2s_joint_grid.restype = WorldId
        S.b2s_many_pyramids.argtypes = [C.c_int, C.c_int, C.c_int]
        S.b2s_many_pyramids.restype = WorldId
        S.b2s_shape_pile.argtypes = [C.c_int, C.c_uint64]
        S.b2s_shape_pile.restype = WorldId
        S.b2s_joint_hub.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64]
        S.b2s_joint_hub.restype = WorldId
        S.b2s_joint_chains.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64]
        S.b2s_joint_chains.restype = WorldId
        S.b2s_joint_zoo.argtypes = [C.c_int, C.c_int, C.c_uint64]
        S.b2s_joint_zoo.restype = WorldId
        S.b2s_chain_scene.argtypes = [C.c_int, C.c_uint64]
        S.b2s_chain_scene.restype = WorldId
        S.b2s_event_scene.argtypes = [C.c_int, C.c_uint64]
        S.b2s_event_scene.restype = WorldId
        S.b2s_empty_world.argtypes = []
        S.b2s_empty_world.restype = WorldId
        S.b2s_add_body.argtypes = [WorldId, C.c_int]
        S.b2s_add_body.restype = BodyId
        S.b2s_add_square.argtypes = [WorldId, C.c_float]
        S.b2s_add_square.restype = BodyId
        S.b2s_destruction.argtypes = []
        S.b2s_destruction.restype = WorldId
        S.b2s_destruction_step.argtypes = [WorldId, C.c_int]
        S.b2s_destruction_step.restype = None
        S.b2s_fast_shots.argtypes = [C.c_int, C.c_uint64]
        S.b2s_fast_shots.restype = WorldId
        S.b2s_sleep_scene.argtypes = []
        S.b2s_sleep_scene.restype = WorldId
        S.b2s_sleep_step.argtypes = [WorldId, C.c_int]
        S.b2s_sleep_step.restype = None
        S.b2s_draw_ints.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_void_p]
        S.b2s_draw_ints.restype = None
        S.b2s_draw_uniform.argtypes = [C.c_int, C.c_uint64, C.c_float, C.c_float, C.c_void_p]
        S.b2s_draw_uniform.restype = None
        S.b2s_draw_normal.argtypes = [C.c_int, C.c_uint64, C.c_void_p]
        S.b2s_draw_normal.restype = None

    # -- scenes --------------------------------------------------------------------
    def pyramid(self, base: int, jitter: float = 0.0, seed: int = 0) -> WorldId:
        w = self.scenes.b2s_pyramid(base, jitter, seed)
        if w.index1 == 0:
            raise RuntimeError(f"{self.name}: world creation failed")
        return w

    def tumbler(self, count: int = 2000, seed: int = 1236, variant: int = 0) -> WorldId:
        return self.scenes.b2s_tumbler(count, seed, variant)

    def drop_boxes(self, heights, vx, vy, friction: float, kinds=None) -> WorldId:
        """Bodies dropped on a ground; kinds[k] picks body k's shape (0 box, 1 circle, 2 capsule)."""
        h = np.ascontiguousarray(heights, np.float32)
        a = np.ascontiguousarray(vx, np.float32)
        b = np.ascontiguousarray(vy, np.float32)
        if kinds is None:
            return self.scenes.b2s_drop_boxes(len(h), h.ctypes.data, a.ctypes.data, b.ctypes.data, friction)
        k = np.ascontiguousarray(kinds, np.int32)
        return self.scenes.b2s_drop_shapes(len(h), h.ctypes.data, a.ctypes.data, b.ctypes.data, friction, k.ctypes.data)

    def hello_world(self):
        body = BodyId()
        w = self.scenes.b2s_hello_world(C.byref(body))
        return w, body

    def tilted_stacks(self) -> WorldId:
        return self.scenes.b2s_tilted_stacks()

    def joint_grid(self, n: int = 100, gravity_y: float = 0.0) -> WorldId:
        return self._made(self.scenes.b2s_joint_grid(n, gravity_y))

    def many_pyramids(self, rows: int = 20, columns: int = 20, base: int = 10) -> WorldId:
        return self._made(self.scenes.b2s_many_pyramids(rows, columns, base))

    def shape_pile(self, count: int = 600, seed: int = 1239) -> WorldId:
        return self._made(self.scenes.b2s_shape_pile(count, seed))

    def joint_hub(self, spokes: int = 20, chains: int = 6, flags: int = 0, seed: int = 1240) -> WorldId:
        """flags: 1 joint limits, 2 joint springs, 4 motors."""
        return self._made(self.scenes.b2s_joint_hub(spokes, chains, flags, seed))

    def joint_chains(self, chains: int = 8, links: int = 8, flags: int = 7, seed: int = 1242) -> WorldId:
        """flags: 1 joint limits, 2 joint springs, 4 motors."""
        return self._made(self.scenes.b2s_joint_chains(chains, links, flags, seed))

    def chain_scene(self, count: int = 200, seed: int = 1260) -> WorldId:
        """Chains: terrain and a bowl of smooth segments with mixed bodies and bullets."""
        return self._made(self.scenes.b2s_chain_scene(count, seed))

    def joint_zoo(self, copies: int = 2, flags: int = 0, seed: int = 1250) -> WorldId:
        """Every joint type: ropes, pendulum, elevators, car, welds, motor and mouse joints, an overflowing spider."""
        return self._made(self.scenes.b2s_joint_zoo(copies, flags, seed))

    def event_scene(self, count: int = 40, seed: int = 1243) -> WorldId:
        return self._made(self.scenes.b2s_event_scene(count, seed))

    def events(self, world: WorldId):
        """The last step's events as plain tuples: (begin, end, hit, sensorBegin, sensorEnd);
        shape ids as (index1, revision), hit events with point, normal and speed bits."""
        L = self.lib
        ce = L.b2World_GetContactEvents(world)
        se = L.b2World_GetSensorEvents(world)
        sid = lambda s: (s.index1, s.revision)
        begin = [(sid(ce.beginEvents[i].shapeIdA), sid(ce.beginEvents[i].shapeIdB)) for i in range(ce.beginCount)]
        end = [(sid(ce.endEvents[i].shapeIdA), sid(ce.endEvents[i].shapeIdB)) for i in range(ce.endCount)]
        f = lambda x: np.float32(x).view(np.uint32).item()
        hit = [(sid(h.shapeIdA), sid(h.shapeIdB), f(h.point.x), f(h.point.y), f(h.normal.x), f(h.normal.y), f(h.approachSpeed))
               for h in (ce.hitEvents[i] for i in range(ce.hitCount))]
        sb = [(sid(se.beginEvents[i].shapeIdA), sid(se.beginEvents[i].shapeIdB)) for i in range(se.beginCount)]
        sn = [(sid(se.endEvents[i].shapeIdA), sid(se.endEvents[i].shapeIdB)) for i in range(se.endCount)]
        return begin, end, hit, sb, sn

    def destruction(self) -> WorldId:
        return self._made(self.scenes.b2s_destruction())

    def destruction_step(self, world: WorldId, step: int) -> None:
        self.scenes.b2s_destruction_step(world, step)

    def sleep_scene(self) -> WorldId:
        """Islands and sleep: resting piles, a chain, bodies created asleep, scripted wakes."""
        return self._made(self.scenes.b2s_sleep_scene())

    def sleep_step(self, world: WorldId, step: int) -> None:
        self.scenes.b2s_sleep_step(world, step)

    def fast_shots(self, count: int = 60, seed: int = 1241) -> WorldId:
        return self._made(self.scenes.b2s_fast_shots(count, seed))

    def _made(self, w: WorldId) -> WorldId:
        if w.index1 == 0:
            raise RuntimeError(f"{self.name}: world creation failed")
        return w

    def draw_ints(self, n, seed, lo, hi):
        out = np.zeros(n, np.int32)
        self.scenes.b2s_draw_ints(n, seed, lo, hi, out.ctypes.data)
        return out

    def draw_uniform(self, n, seed, lo, hi):
        out = np.zeros(n, np.float32)
        self.scenes.b2s_draw_uniform(n, seed, lo, hi, out.ctypes.data)
        return out

    def draw_normal(self, n, seed):
        out = np.zeros(n, np.float32)
        self.scenes.b2s_draw_normal(n, seed, out.ctypes.data)
        return out

    # -- stepping and state ----------------------------------------------------------
    def step(self, world: WorldId, dt: float = 1.0 / 60.0, substeps: int = 4, count: int = 1):
        for _ in range(count):
            self.lib.b2World_Step(world, dt, substeps)

    def destroy(self, world: WorldId):
        self.lib.b2DestroyWorld(world)

    def counters(self, world: WorldId) -> Counters:
        return self.lib.b2World_GetCounters(world)

    def bodies(self, world: WorldId) -> np.ndarray:
        n = self.lib.b2World_InspectBodies(world, None, 0)
        out = np.zeros((n, BODY_FLOATS), np.float32)
        self.lib.b2World_InspectBodies(world, out.ctypes.data, n)
        return out

    def shapes(self, world: WorldId) -> np.ndarray:
        n = self.lib.b2World_InspectShapes(world, None, 0)
        arr = (InspectShape * max(n, 1))()
        self.lib.b2World_InspectShapes(world, C.addressof(arr), n)
        return np.ctypeslib.as_array(arr)[:n].copy() if n else np.zeros(0, dtype=np.dtype(InspectShape))

    def islands(self, world: WorldId) -> np.ndarray:
        """(solver set, island id) per body id; -1 for free slots."""
        n = self.lib.b2World_InspectIslands(world, None, 0)
        out = np.zeros((n, 2), np.int32)
        self.lib.b2World_InspectIslands(world, out.ctypes.data, n)
        return out

    def contacts(self, world: WorldId) -> np.ndarray:
        n = self.lib.b2World_InspectContacts(world, None, 0)
        arr = (InspectContact * max(n, 1))()
        self.lib.b2World_InspectContacts(world, C.addressof(arr), n)
        return np.ctypeslib.as_array(arr)[:n].copy() if n else np.zeros(0, dtype=np.dtype(InspectContact))


def contact_table(contacts: np.ndarray) -> np.ndarray:
    """(contactId, shapeIdA, shapeIdB, colorIndex, touching, pointCount) rows."""
    if len(contacts) == 0:
        return np.zeros((0, 6), np.int64)
    return np.stack([contacts["contactId"], contacts["shapeIdA"], contacts["shapeIdB"],
                     contacts["colorIndex"], contacts["touching"], contacts["pointCount"]], 1).astype(np.int64)


def finite_max_rel(a: np.ndarray, b: np.ndarray, floor: float = 1.0) -> float:
    """max |a-b| / max(|b|, floor) over finite entries."""
    m = np.isfinite(a) & np.isfinite(b)
    if not m.any():
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.maximum(np.abs(b[m]), floor)))


__all__ = ["Vec2", "Rot", "Transform", "WorldId", "BodyId", "Counters", "Profile",
           "InspectContact", "InspectShape", "InspectPoint", "Backend", "contact_table",
           "finite_max_rel", "BODY_FLOATS", "math"]


class ManifoldPoint(C.Structure):
    _fields_ = [("point", Vec2), ("anchorA", Vec2), ("anchorB", Vec2), ("separation", C.c_float),
                ("normalImpulse", C.c_float), ("tangentImpulse", C.c_float),
                ("maxNormalImpulse", C.c_float), ("normalVelocity", C.c_float),
                ("id", C.c_uint16), ("persisted", C.c_bool)]


class Manifold(C.Structure):
    _fields_ = [("points", ManifoldPoint * 2), ("normal", Vec2), ("pointCount", C.c_int32)]


MANIFOLD_BYTES = C.sizeof(Manifold)


class ContactSolveDesc(C.Structure):
    """include/box2d/gpu.h b2ContactSolveDesc."""
    _fields_ = [("states", C.c_void_p), ("massData", C.c_void_p), ("forces", C.c_void_p),
                ("damping", C.c_void_p), ("bodies", C.c_void_p), ("bodyCount", C.c_int32),
                ("contactBodies", C.c_void_p), ("contactMix", C.c_void_p), ("manifolds", C.c_void_p),
                ("contactCount", C.c_int32), ("colorStart", C.c_int32 * 13),
                ("timeStep", C.c_float), ("subStepCount", C.c_int32), ("gravity", Vec2),
                ("contactHertz", C.c_float), ("contactDampingRatio", C.c_float),
                ("contactPushout", C.c_float), ("restitutionThreshold", C.c_float),
                ("enableWarmStarting", C.c_bool), ("stream", C.c_void_p)]


def bind_solve_api(lib: C.CDLL) -> None:
    lib.b2SolveContacts.argtypes = [C.POINTER(ContactSolveDesc)]
    lib.b2SolveContacts.restype = C.c_int


class DeviceTimes(C.Structure):
    """include/box2d/gpu.h b2DeviceTimes."""
    _fields_ = [("step", C.c_float), ("collide", C.c_float), ("solve", C.c_float), ("finalize", C.c_float),
                ("eventCount", C.c_int), ("recordCount", C.c_int), ("launches", C.c_int), ("fusedSolver", C.c_int),
                ("hostToDeviceBytes", C.c_longlong), ("deviceToHostBytes", C.c_longlong),
                ("hostPairQuery", C.c_float), ("hostPairRules", C.c_float), ("hostContactCreate", C.c_float),
                ("hostEvents", C.c_float), ("hostSolveLists", C.c_float), ("hostTreeRebuild", C.c_float),
                ("hostRecords", C.c_float), ("hostContinuous", C.c_float)]


def bind_gpu_api(lib: C.CDLL) -> None:
    """Binds the additive device entry points of include/box2d/gpu.h."""
    lib.b2World_GetStatus.argtypes = [WorldId]
    lib.b2World_GetStatus.restype = C.c_int
    lib.b2World_GetToiEventCount.argtypes = [WorldId]
    lib.b2World_GetToiEventCount.restype = C.c_int
    lib.b2World_EnableDeviceTiming.argtypes = [WorldId, C.c_bool]
    lib.b2World_EnableDeviceTiming.restype = None
    lib.b2World_GetDeviceTimes.argtypes = [WorldId]
    lib.b2World_GetDeviceTimes.restype = DeviceTimes
    lib.b2World_EnableFusedSolver.argtypes = [WorldId, C.c_bool]
    lib.b2World_EnableFusedSolver.restype = None
    lib.b2World_GetBodyStates.argtypes = [WorldId, C.c_void_p, C.c_int]
    lib.b2World_GetBodyStates.restype = C.c_int


class BatchStats(C.Structure):
    """include/box2d/gpu.h b2BatchStats."""
    _fields_ = [("collide", C.c_float), ("solve", C.c_float), ("solveThreads", C.c_int), ("launches", C.c_int),
                ("hostBegin", C.c_float), ("hostCollide", C.c_float), ("hostMiddle", C.c_float),
                ("hostSolve", C.c_float), ("hostFinish", C.c_float), ("hostThreads", C.c_int),
                ("solveCtasPerSm", C.c_int)]


def bind_batch_api(lib: C.CDLL) -> None:
    lib.b2World_StepBatch.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_int]
    lib.b2World_StepBatch.restype = None
    lib.b2World_GetBatchStats.argtypes = []
    lib.b2World_GetBatchStats.restype = BatchStats


def world_array(worlds) -> C.Array:
    """A C array of b2WorldId for b2World_StepBatch."""
    arr = (WorldId * len(worlds))()
    for i, w in enumerate(worlds):
        arr[i] = w
    return arr
