"""The plain-C oracle against the reference: known answers from the reference's own
unit tests, golden vectors produced by the reference build, and (where the reference
sources are present) step-by-step lockstep with the reference itself."""
import ctypes as C
import hashlib
import math
import os

import numpy as np
import pytest

from box2c_gb300.capi import Vec2, Transform, Rot, contact_table
from tests.golden.make_golden import SCENES, make_scene, digest, step_scene
from tests.golden.shapes import Manifold, random_pairs, manifold_array
from tests.helpers import lockstep, run_world_api_checks

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FLT_EPS = float(np.finfo(np.float32).eps)


class SegDist(C.Structure):
    _fields_ = [("closest1", Vec2), ("closest2", Vec2), ("fraction1", C.c_float), ("fraction2", C.c_float),
                ("distanceSquared", C.c_float)]


def test_segment_distance_kat(oracle):
    # reference test/test_distance.c:11-29
    f = oracle.lib.b2SegmentDistance
    f.restype = SegDist
    f.argtypes = [Vec2, Vec2, Vec2, Vec2]
    r = f(Vec2(-1, -1), Vec2(-1, 1), Vec2(2, 0), Vec2(1, 0))
    assert abs(r.fraction1 - 0.5) <= FLT_EPS and abs(r.fraction2 - 1.0) <= FLT_EPS
    assert abs(r.closest1.x + 1) <= FLT_EPS and abs(r.closest1.y) <= FLT_EPS
    assert abs(r.closest2.x - 1) <= FLT_EPS and abs(r.closest2.y) <= FLT_EPS
    assert abs(r.distanceSquared - 4) <= FLT_EPS


class MassData(C.Structure):
    _fields_ = [("mass", C.c_float), ("center", Vec2), ("rotationalInertia", C.c_float)]


def test_mass_kat(oracle):
    # reference test/test_shape.c:18-70: circle at (1,0) r=1, box 1x1 half extents
    from tests.golden.shapes import Circle, _box
    L = oracle.lib
    L.b2ComputeCircleMass.restype = MassData
    L.b2ComputeCircleMass.argtypes = [C.c_void_p, C.c_float]
    c = Circle(Vec2(1.0, 0.0), 1.0)
    md = L.b2ComputeCircleMass(C.addressof(c), 1.0)
    assert abs(np.float32(md.mass) - np.float32(math.pi)) <= FLT_EPS
    assert md.center.x == 1.0 and md.center.y == 0.0
    assert abs(np.float32(md.rotationalInertia) - np.float32(1.5) * np.float32(math.pi)) <= FLT_EPS
    L.b2ComputePolygonMass.restype = MassData
    L.b2ComputePolygonMass.argtypes = [C.c_void_p, C.c_float]
    box = _box(1.0, 1.0)
    md = L.b2ComputePolygonMass(C.addressof(box), 1.0)
    assert abs(md.mass - 4.0) <= FLT_EPS
    assert abs(md.center.x) <= FLT_EPS and abs(md.center.y) <= FLT_EPS
    assert abs(np.float32(md.rotationalInertia) - np.float32(8.0) / np.float32(3.0)) <= 2 * FLT_EPS


def test_manifold_golden(oracle):
    golden = np.load(os.path.join(GOLDEN, "manifolds.npz"))["outputs"]
    pairs = random_pairs(seed=7, count=len(golden))
    for k, (kind, a, xa, b, xb) in enumerate(pairs):
        fn = getattr(oracle.lib, kind)
        fn.restype = Manifold
        fn.argtypes = [C.c_void_p, Transform, C.c_void_p, Transform]
        got = manifold_array(fn(C.addressof(a), xa, C.addressof(b), xb))
        assert np.array_equal(got.view(np.uint32), golden[k].view(np.uint32)), (k, kind, got, golden[k])


@pytest.mark.parametrize("name", list(SCENES))
def test_scene_golden(oracle, name):
    """Per-step bit-exact body state, contact table and solver sets / island ids against
    the reference's hashes."""
    g = np.load(os.path.join(GOLDEN, "scenes.npz"))
    steps, snaps = SCENES[name]
    bh, ch, ih = g[f"{name}/body_hash"], g[f"{name}/contact_hash"], g[f"{name}/island_hash"]
    w = make_scene(oracle, name)
    try:
        for s in range(steps + 1):
            bodies = oracle.bodies(w)
            assert digest(contact_table(oracle.contacts(w))) == ch[s], f"{name}: contact table differs at step {s}"
            assert digest(oracle.islands(w)) == ih[s], f"{name}: solver sets / islands differ at step {s}"
            if digest(bodies.view(np.uint32)) != bh[s]:
                pytest.fail(f"{name}: body state differs at step {s}")
            if s in snaps:
                assert np.array_equal(bodies.view(np.uint32), g[f"{name}/bodies_{s}"].view(np.uint32))
            if s < steps:
                step_scene(oracle, name, w, s + 1)
    finally:
        oracle.destroy(w)


def test_hello_world(oracle):
    # reference test/test_world.c:17-97
    w, body = oracle.hello_world()
    oracle.step(w, count=90)
    p = oracle.lib.b2Body_GetPosition(body)
    q = oracle.lib.b2Body_GetRotation(body)
    oracle.destroy(w)
    assert abs(p.x) < 0.01 and abs(p.y - 1.0) < 0.01 and abs(math.atan2(q.s, q.c)) < 0.01


def test_determinism_repeat(oracle):
    # reference test/test_determinism.c:179-202: the same scene twice is bit-identical
    finals = []
    for _ in range(2):
        w = oracle.tilted_stacks()
        oracle.step(w, dt=1 / 60, substeps=3, count=100)
        finals.append(oracle.bodies(w).copy())
        oracle.destroy(w)
    assert np.array_equal(finals[0].view(np.uint32), finals[1].view(np.uint32))


@pytest.mark.parametrize("scene,steps", [("pyramid20", 120), ("tumbler", 120), ("tumbler_ref", 60), ("tilted", 100)])
def test_lockstep_reference(oracle, reference, scene, steps):
    make = {
        "pyramid20": lambda b: b.pyramid(20),
        "tumbler": lambda b: b.tumbler(1200, 99, 0),
        "tumbler_ref": lambda b: b.tumbler(0, 0, 1),
        "tilted": lambda b: b.tilted_stacks(),
    }[scene]
    step, detail, _ = lockstep(reference, oracle, make, steps, check_manifolds=True)
    assert step is None, f"{scene}: {detail} at step {step}"


def test_fp64_oracle_tracks_fp32(oracle, oracle64):
    """The FP64 build runs the same step; on a short drop it stays within 1e-4 of FP32."""
    h = [1.2, 2.0, 3.1, 4.5]
    w32 = oracle.drop_boxes(h, [0.3, -0.2, 0.1, 0.0], [0.0, 0.5, -1.0, 0.2], 0.6)
    w64 = oracle64.drop_boxes(h, [0.3, -0.2, 0.1, 0.0], [0.0, 0.5, -1.0, 0.2], 0.6)
    oracle.step(w32, count=30)
    oracle64.step(w64, count=30)
    a, b = oracle.bodies(w32), oracle64.bodies(w64)
    oracle.destroy(w32)
    oracle64.destroy(w64)
    assert np.nanmax(np.abs(a[:, :2] - b[:, :2])) < 1e-3


@pytest.mark.parametrize("scene,steps", [("pyramid_jitter", 60), ("tumbler", 60)])
def test_threaded_oracle_is_bit_identical(oracle, scene, steps):
    """The oracle's parallel loops (colour rows, bodies, narrowphase contacts; the CPU
    baselines use them) give the bits of the serial oracle."""
    make = {"pyramid_jitter": lambda: oracle.pyramid(40, 0.01, 77), "tumbler": lambda: oracle.tumbler(900, 5, 0)}[scene]
    L = oracle.lib
    L.b2o_SetThreads.argtypes = [C.c_int]
    L.b2o_SetThreads.restype = C.c_int
    states = []
    try:
        for threads in (1, 8):
            L.b2o_SetThreads(threads)
            w = make()
            oracle.step(w, count=steps)
            states.append((oracle.bodies(w).view(np.uint32).copy(), contact_table(oracle.contacts(w))))
            oracle.destroy(w)
    finally:
        L.b2o_SetThreads(1)
    assert np.array_equal(states[0][0], states[1][0])
    assert np.array_equal(states[0][1], states[1][1])


@pytest.mark.parametrize("scene", ["joint_chains", "joint_hub_limits"])
def test_own_atan2_per_step_error_and_drift(reference, oracle_atan, scene):
    """Joint springs and limits take the joint angle through atan2; the library (and the
    oracle build it is checked against bit for bit) uses its own atan2, within one float
    ulp of the reference's atan2f.  From identical states the first step's error is the
    per-step error: within 1e-5 relative (max(|ref|, 1) as the scale).  The drift after
    N steps is reported; in these many-body scenes a one-ulp difference grows."""
    make = {"joint_chains": lambda b: b.joint_chains(8, 8, 7, 1242),
            "joint_hub_limits": lambda b: b.joint_hub(20, 6, 7, 1240)}[scene]
    wr, wa = make(reference), make(oracle_atan)
    drift = {}
    try:
        for s in range(1, 301):
            reference.step(wr)
            oracle_atan.step(wa)
            if s in (1, 10, 60, 300):
                a, b = oracle_atan.bodies(wa), reference.bodies(wr)
                drift[s] = float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))
    finally:
        reference.destroy(wr)
        oracle_atan.destroy(wa)
    print(f"{scene}: max rel state error after N steps {drift}")
    assert drift[1] <= 1e-5, drift
    assert all(np.isfinite(v) for v in drift.values())


def test_destruction_lockstep_reference(reference, oracle):
    """b2DestroyBody / b2DestroyShape / b2DestroyJoint mid-run (pyramid bodies, joints in
    the colours and in the overflow set, one shape of multi-shape bodies, a jointed hub,
    a static shape; then new bodies on the freed ids): the oracle stays bit-identical to
    the reference every step, manifolds included."""
    step, detail, _ = lockstep(oracle, reference, lambda b: b.destruction(), 160, check_manifolds=True,
                               after_step=lambda b, w, s: b.destruction_step(w, s))
    assert step is None, f"{detail} at step {step}"


def test_sleep_lockstep_reference(reference, oracle):
    """Islands and sleep (reference src/island.c, src/solver_set.c): piles and a damped
    chain fall asleep island by island, two bodies created asleep share a set through a
    joint, and a destroyed body and joint, a dropped box, a rolled ball, a velocity set on
    a sleeping body, SetAwake and the body and world sleep switches wake them.  Every
    step the body states, the contact table and every body's solver set and island id
    equal the reference's."""
    step, detail, _ = lockstep(oracle, reference, lambda b: b.sleep_scene(), 360, check_manifolds=True,
                               after_step=lambda b, w, s: b.sleep_step(w, s), check_islands=True)
    assert step is None, f"{detail} at step {step}"


def test_hello_world_sleeps_like_reference(reference, oracle):
    """Reference test/test_world.c:17-97 with sleep on: the box's island falls asleep at
    step 88 in both, in set 3 of island 0, and stays there."""
    step, detail, _ = lockstep(oracle, reference, lambda b: b.hello_world()[0], 200, check_islands=True)
    assert step is None, f"{detail} at step {step}"
    w = oracle.hello_world()[0]
    oracle.step(w, count=88)
    assert oracle.islands(w).tolist() == [[0, -1], [3, 0]]
    oracle.destroy(w)


@pytest.mark.parametrize("backend", ["reference", "oracle"])
def test_world_destroy_all_bodies_and_validity(request, backend):
    """Reference test/test_world.c:121-204 (DestroyAllBodiesWorld, TestIsValid) restated
    over the C API."""
    run_world_api_checks(request.getfixturevalue(backend))


def test_events_match_reference(reference, oracle):
    """Contact begin/end touch events, hit events and sensor begin/end overlap events of
    every step, in order, equal the reference's (reference src/world.c:540-662,
    src/solver.c:1670-1723, src/contact.c:476-503); the state stays bit-identical."""
    wo, wr = oracle.event_scene(40, 1243), reference.event_scene(40, 1243)
    totals = [0] * 5
    try:
        for s in range(1, 301):
            oracle.step(wo)
            reference.step(wr)
            eo, er = oracle.events(wo), reference.events(wr)
            assert eo == er, f"events differ at step {s}"
            totals = [t + len(e) for t, e in zip(totals, er)]
    finally:
        oracle.destroy(wo)
        reference.destroy(wr)
    assert all(t > 0 for t in totals), totals
    step, detail, _ = lockstep(oracle, reference, lambda b: b.event_scene(40, 1243), 300, check_manifolds=True)
    assert step is None, f"{detail} at step {step}"


def joint_api_script(backend):
    """Runs the joint API script (every joint type's creation, queries and setters; see
    b2s_joint_api_script) on a backend; returns its outputs as float32."""
    f = backend.scenes.b2s_joint_api_script
    f.argtypes = [C.POINTER(C.c_float), C.c_int]
    f.restype = C.c_int
    out = (C.c_float * 4096)()
    n = f(out, 4096)
    assert 0 < n <= 4096
    return np.array(out[:n], np.float32)


def test_joint_api_script_matches_reference(reference, oracle):
    """Every joint type's creation (clamped and reordered limits, normalised axes),
    queries, reaction forces and torques, setters that reset accumulated impulses,
    collide-connected toggles and destruction: the oracle gives the reference's bits."""
    a, b = joint_api_script(oracle), joint_api_script(reference)
    assert a.shape == b.shape
    bad = np.nonzero(a.view(np.uint32) != b.view(np.uint32))[0]
    assert bad.size == 0, (bad[:10], a[bad[:10]], b[bad[:10]])


@pytest.mark.parametrize("copies,flags", [(2, 0), (3, 1)])
def test_joint_zoo_lockstep_reference(reference, oracle, copies, flags):
    """Every joint type with contacts, in the colours and in the overflow colour: the
    oracle stays bit-identical to the reference every step, manifolds included."""
    step, detail, _ = lockstep(reference, oracle, lambda b: b.joint_zoo(copies, flags, 1250 + flags), 200,
                               check_manifolds=True)
    assert step is None, f"{detail} at step {step}"


def test_smooth_segment_manifolds_golden(oracle):
    """The oracle's chain-link manifolds against the reference's golden vectors."""
    from tests.golden.shapes import collide_smooth, random_smooth_pairs
    golden = np.load(os.path.join(GOLDEN, "smooth_manifolds.npz"))["outputs"]
    for k, entry in enumerate(random_smooth_pairs(seed=11, count=len(golden))):
        got = collide_smooth(oracle.lib, entry)
        assert np.array_equal(got.view(np.uint32), golden[k].view(np.uint32)), (k, entry[0])


def test_chain_scene_lockstep_reference(reference, oracle):
    """Chains (open terrain and a closed bowl of smooth segments) against circles,
    capsules, boxes and rounded boxes, with fast bodies and bullets: bit-identical every
    step, manifolds included."""
    step, detail, _ = lockstep(reference, oracle, lambda b: b.chain_scene(200, 1260), 300, check_manifolds=True)
    assert step is None, f"{detail} at step {step}"
