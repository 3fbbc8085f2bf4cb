"""GPU pipeline against the plain-C oracle (and the reference's golden vectors): pair
sets, colours, manifolds and body state must be bit-identical every step."""
import math
import os

import numpy as np
import pytest

from box2c_gb300.capi import bind_gpu_api, contact_table
from tests.golden.make_golden import SCENES, make_scene, digest, step_scene
from tests.helpers import lockstep

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", ["pyramid20", "tilted", "hello", "tumbler2000", "pyramid100", "joint_grid30",
                                  "joint_grid100", "many_pyramids5", "many_pyramids20", "shape_pile", "joint_hub",
                                  "fast_shots", "chain_scene", "sleep_scene"])
def test_gpu_matches_reference_golden(gpu, name):
    g = np.load(os.path.join(GOLDEN, "scenes.npz"))
    steps, snaps = SCENES[name]
    bh, ch, ih = g[f"{name}/body_hash"], g[f"{name}/contact_hash"], g[f"{name}/island_hash"]
    w = make_scene(gpu, name)
    try:
        for s in range(steps + 1):
            assert digest(contact_table(gpu.contacts(w))) == ch[s], f"{name}: pairs/colours differ at step {s}"
            assert digest(gpu.islands(w)) == ih[s], f"{name}: solver sets / islands differ at step {s}"
            bodies = gpu.bodies(w)
            if s in snaps:
                ref = g[f"{name}/bodies_{s}"]
                m = np.isfinite(ref)
                rel = np.max(np.abs(bodies[m] - ref[m]) / np.maximum(np.abs(ref[m]), 1.0))
                assert rel <= 1e-5, f"{name}: step {s} max rel err {rel}"
            assert digest(bodies.view(np.uint32)) == bh[s], f"{name}: body state not bit-exact at step {s}"
            if s < steps:
                step_scene(gpu, name, w, s + 1)
    finally:
        gpu.destroy(w)


def test_gpu_sleep_lockstep_oracle(gpu, oracle):
    """Islands and sleep on the device path: sleeping bodies leave the awake list and the
    integration, their contacts leave the narrowphase, a woken set rejoins the solve in
    the step that woke it (contact begin, destruction, velocity, SetAwake, the sleep
    switches) with the identity state.  Body states, manifolds, contact table, solver
    sets and island ids equal the oracle's every step."""
    step, detail, _ = lockstep(gpu, oracle, lambda b: b.sleep_scene(), 360, check_manifolds=True,
                               after_step=lambda b, w, s: b.sleep_step(w, s), check_islands=True)
    assert step is None, f"{detail} at step {step}"


@pytest.mark.parametrize("scene,steps,sub", [
    ("pyramid20", 300, 4), ("tumbler", 150, 4), ("tumbler_grid", 100, 4), ("tilted", 100, 3),
    ("pyramid_jitter", 120, 4), ("drop", 120, 4)])
def test_gpu_lockstep_oracle(gpu, oracle, scene, steps, sub):
    make = {
        "pyramid20": lambda b: b.pyramid(20),
        "pyramid_jitter": lambda b: b.pyramid(30, 0.01, 77),
        "tumbler": lambda b: b.tumbler(900, 5, 0),
        "tumbler_grid": lambda b: b.tumbler(0, 0, 1),
        "tilted": lambda b: b.tilted_stacks(),
        "drop": lambda b: b.drop_boxes([1.0, 2.5, 4.0, 1.7, 3.3, 2.2, 4.8, 1.1],
                                       [0.4, -0.3, 1.2, -0.9, 0.0, 0.5, -0.2, 0.8],
                                       [0.1, -1.0, 0.3, 0.0, 0.7, -0.4, 0.2, 1.5], 0.45),
    }[scene]
    step, detail, worst = lockstep(gpu, oracle, make, steps, substeps=sub, check_manifolds=True)
    assert step is None, f"{scene}: {detail} at step {step}"


@pytest.mark.parametrize("scene,steps", [("shape_pile", 250), ("joint_hub_motors", 250), ("fast_shots", 150),
                                         ("many_pyramids", 100), ("joint_grid", 100), ("chains", 300)])
def test_gpu_lockstep_oracle_new_paths(gpu, oracle, scene, steps):
    """Device paths the pyramid and tumbler scenes do not reach, stepped against the oracle
    with every manifold compared: capsule and segment manifolds (capsule-capsule,
    polygon-capsule, segment-polygon, segment-capsule, segment-circle) and rounded
    polygons; revolute joints in the graph colours and in the overflow colour, with
    motors; time of impact of fast bodies and bullets; segment grounds; chains of smooth
    segments (one-sided links with ghost vertices, the contact's closest-feature cache,
    the continuous-collision rule for links)."""
    make = {
        "chains": lambda b: b.chain_scene(160, 94),
        "shape_pile": lambda b: b.shape_pile(300, 91),
        "joint_hub_motors": lambda b: b.joint_hub(16, 4, 4, 92),
        "fast_shots": lambda b: b.fast_shots(40, 93),
        "many_pyramids": lambda b: b.many_pyramids(3, 3, 10),
        "joint_grid": lambda b: b.joint_grid(20, -10.0),
    }[scene]
    step, detail, worst = lockstep(gpu, oracle, make, steps, check_manifolds=True)
    assert step is None, f"{scene}: {detail} at step {step}"


def test_gpu_time_of_impact_events(gpu, oracle):
    """Continuous collision happens on the device path as often as in the oracle: the
    projectiles stop at the thin wall instead of tunnelling through it."""
    import ctypes as C
    from box2c_gb300.capi import WorldId
    bind_gpu_api(gpu.lib)
    oracle.lib.b2o_ToiEventCount.argtypes = [WorldId]
    oracle.lib.b2o_ToiEventCount.restype = C.c_int
    wg, wo = gpu.fast_shots(60, 1241), oracle.fast_shots(60, 1241)
    gpu.step(wg, count=120)
    oracle.step(wo, count=120)
    ng, no = gpu.lib.b2World_GetToiEventCount(wg), oracle.lib.b2o_ToiEventCount(wo)
    bg = gpu.bodies(wg)
    gpu.destroy(wg)
    oracle.destroy(wo)
    assert ng == no and ng > 50
    # no projectile tunnelled through the wall (x = 20, 0.05 thick); rows are
    # p.x p.y q.c q.s v.x v.y w type, static bodies included
    dynamic = bg[:, 7] == 2
    assert np.all(bg[dynamic, 0] < 20.0)


def test_gpu_hello_world(gpu):
    # reference test/test_world.c:17-97 acceptance bounds
    w, body = gpu.hello_world()
    gpu.step(w, count=90)
    p = gpu.lib.b2Body_GetPosition(body)
    q = gpu.lib.b2Body_GetRotation(body)
    gpu.destroy(w)
    assert abs(p.x) < 0.01 and abs(p.y - 1.0) < 0.01 and abs(math.atan2(q.s, q.c)) < 0.01


def test_gpu_large_pyramid_full_size(gpu, oracle):
    """Full-size workload (100 rows, 5050 boxes, 500 steps): the GPU state equals the
    oracle's bit for bit at the end; counts and colours match; nothing is NaN."""
    wg, wo = gpu.pyramid(100, 0.01, 1235), oracle.pyramid(100, 0.01, 1235)
    gpu.step(wg, count=500)
    oracle.step(wo, count=500)
    cg, co = gpu.counters(wg), oracle.counters(wo)
    bg, bo = gpu.bodies(wg), oracle.bodies(wo)
    tg, to = contact_table(gpu.contacts(wg)), contact_table(oracle.contacts(wo))
    gpu.destroy(wg)
    oracle.destroy(wo)
    assert cg.bodyCount == 5051 and list(cg.colorCounts) == list(co.colorCounts)
    assert np.isfinite(bg).all()
    assert np.array_equal(tg, to)
    assert np.array_equal(bg.view(np.uint32), bo.view(np.uint32))


def _per_phase(gpu, world):
    bind_gpu_api(gpu.lib)
    gpu.lib.b2World_EnableFusedSolver(world, False)
    return world


@pytest.mark.parametrize("scene,steps,sub", [("pyramid20", 150, 4), ("tumbler", 100, 4), ("tilted", 60, 3)])
def test_gpu_per_phase_solver_lockstep_oracle(gpu, oracle, scene, steps, sub):
    """The one-launch-per-phase solver path (used when a world does not fit on chip)."""
    scenes = {
        "pyramid20": lambda b: b.pyramid(20),
        "tumbler": lambda b: b.tumbler(900, 5, 0),
        "tilted": lambda b: b.tilted_stacks(),
    }

    def make(b):
        w = scenes[scene](b)
        return _per_phase(b, w) if b is gpu else w

    step, detail, _ = lockstep(gpu, oracle, make, steps, substeps=sub, check_manifolds=True)
    assert step is None, f"{scene}: {detail} at step {step}"


@pytest.mark.parametrize("fused", [True, False])
def test_gpu_solver_path_selection(gpu, fused):
    """The large pyramid runs its solver stage fused by default; both paths agree."""
    bind_gpu_api(gpu.lib)
    w = gpu.pyramid(100, 0.01, 1235)
    gpu.lib.b2World_EnableFusedSolver(w, fused)
    gpu.step(w, count=3)
    t = gpu.lib.b2World_GetDeviceTimes(w)
    status = gpu.lib.b2World_GetStatus(w)
    gpu.destroy(w)
    assert status == 0
    assert t.fusedSolver == (1 if fused else 0)


@pytest.mark.parametrize("scene", ["joint_chains", "joint_hub_limits"])
def test_gpu_joint_limits_springs_lockstep(gpu, oracle_atan, scene):
    """Revolute joints with limits, springs and motors, against the oracle build that
    uses the library's own atan2 for the joint angle: bit-identical every step (in the
    graph colours and in the overflow colour, with contacts in the hub scene)."""
    make = {"joint_chains": lambda b: b.joint_chains(8, 8, 7, 1242),
            "joint_hub_limits": lambda b: b.joint_hub(20, 6, 7, 1240)}[scene]
    step, detail, worst = lockstep(gpu, oracle_atan, make, 300, check_manifolds=True)
    assert step is None, f"{scene}: {detail} at step {step}"


@pytest.mark.parametrize("copies,flags,steps,per_phase", [(2, 0, 300, False), (3, 1, 200, False), (2, 0, 150, True)])
def test_gpu_joint_zoo_lockstep(gpu, oracle_atan, copies, flags, steps, per_phase):
    """Every joint type (distance, motor, mouse, prismatic, revolute, weld, wheel; springs,
    limits and motors; a hub whose joints of every type overflow the graph colours), with
    contacts, against the oracle build that uses the library's own atan2: bit-identical
    every step, manifolds included, on the fused and on the per-phase solver path."""
    def make(b):
        w = b.joint_zoo(copies, flags, 1250 + flags)
        return _per_phase(b, w) if ( per_phase and b is gpu ) else w

    step, detail, worst = lockstep(gpu, oracle_atan, make, steps, check_manifolds=True)
    assert step is None, f"joint zoo: {detail} at step {step}"


# Positions of b2RevoluteJoint_GetAngle in the joint API script's output (four readouts
# of 120 values; the angle is value 98 of each): the library answers that query on the
# host with the C library's atan2f, as the reference does, so it may differ from the
# own-atan2 oracle build by one float ulp.
_ANGLE_SLOTS = [98 + 120 * k for k in range(4)]


def test_gpu_joint_api_script(gpu, oracle_atan):
    """Every joint type's creation, queries, reaction forces and torques, impulse-resetting
    setters, collide-connected toggles and destruction through the library: the bits of
    the own-atan2 oracle build (the revolute angle query within 2 ulp)."""
    from tests.test_oracle import joint_api_script
    a, b = joint_api_script(gpu), joint_api_script(oracle_atan)
    assert a.shape == b.shape == (514,)
    mask = np.ones(a.shape, bool)
    mask[_ANGLE_SLOTS] = False
    bad = np.nonzero((a.view(np.uint32) != b.view(np.uint32)) & mask)[0]
    assert bad.size == 0, (bad[:10], a[bad[:10]], b[bad[:10]])
    ulps = np.abs(a[_ANGLE_SLOTS].view(np.int32).astype(np.int64) - b[_ANGLE_SLOTS].view(np.int32).astype(np.int64))
    assert ulps.max() <= 2, (a[_ANGLE_SLOTS], b[_ANGLE_SLOTS])


@pytest.mark.parametrize("name", ["joint_chains", "joint_hub_limits", "joint_zoo", "joint_zoo_collide"])
def test_gpu_joint_limits_against_reference_golden(gpu, name):
    """The same scenes against the reference's own states: the first step (identical
    start) within 1e-5 relative; the drift at later snapshots is printed (a one-ulp
    difference of atan2 grows in these many-body scenes)."""
    g = np.load(os.path.join(GOLDEN, "scenes.npz"))
    steps, snaps = SCENES[name]
    w = make_scene(gpu, name)
    drift = {}
    try:
        for s in range(1, steps + 1):
            gpu.step(w)
            if s in snaps:
                ref = g[f"{name}/bodies_{s}"]
                b = gpu.bodies(w)
                drift[s] = float(np.max(np.abs(b - ref) / np.maximum(np.abs(ref), 1.0)))
    finally:
        gpu.destroy(w)
    print(f"{name}: max rel state error vs the reference after N steps {drift}")
    assert drift[1] <= 1e-5, drift
    assert all(np.isfinite(v) for v in drift.values())


def test_gpu_destruction_lockstep_oracle(gpu, oracle):
    """b2DestroyBody / b2DestroyShape / b2DestroyJoint between steps (pyramid bodies,
    joints in the colours and in the overflow set, one shape of two-shape bodies, a hub
    with its joints, a static shape, then new bodies on the freed ids): the device stays
    bit-identical to the oracle, which the CPU tests pin to the reference."""
    step, detail, _ = lockstep(gpu, oracle, lambda b: b.destruction(), 160, check_manifolds=True,
                               after_step=lambda b, w, s: b.destruction_step(w, s))
    assert step is None, f"{detail} at step {step}"


def test_gpu_world_destroy_all_bodies_and_validity(gpu):
    """Reference test/test_world.c:121-204 (DestroyAllBodiesWorld, TestIsValid)."""
    from tests.helpers import run_world_api_checks
    run_world_api_checks(gpu)


def test_gpu_events_match_oracle(gpu, oracle):
    """Contact begin/end, hit and sensor events of every step equal the oracle's (which
    the CPU tests pin to the reference): sensors tested by GJK overlap on the device with
    each contact's closest-feature cache, hit events from the solved manifolds."""
    from box2c_gb300.capi import bind_gpu_api
    bind_gpu_api(gpu.lib)
    wg, wo = gpu.event_scene(40, 1243), oracle.event_scene(40, 1243)
    totals = [0] * 5
    try:
        for s in range(1, 301):
            gpu.step(wg)
            oracle.step(wo)
            eg, eo = gpu.events(wg), oracle.events(wo)
            assert eg == eo, f"events differ at step {s}"
            totals = [t + len(e) for t, e in zip(totals, eo)]
        assert np.array_equal(gpu.bodies(wg).view(np.uint32), oracle.bodies(wo).view(np.uint32))
    finally:
        gpu.destroy(wg)
        oracle.destroy(wo)
    assert all(t > 0 for t in totals), totals
