"""b2SolveContacts (include/box2d/gpu.h) against the oracle's solver stage.

The oracle steps a scene and records what its solver stage (reference src/solver.c
b2SolverStage_PrepareContacts .. b2SolverStage_StoreImpulses) reads and writes: body
velocities and deltas, mass, forces, damping, the awake list, the coloured contacts
with their manifolds.  The same inputs go through b2SolveContacts on the device;
body states and stored impulses must match bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from box2c_gb300.capi import MANIFOLD_BYTES, ContactSolveDesc, Vec2, bind_solve_api

DT, SUBSTEPS = 1.0 / 60.0, 4


class Capture(C.Structure):
    """oracle/b2o_solver.c b2oCapture."""
    _fields_ = [("bodyCap", C.c_int32), ("contactCap", C.c_int32), ("bodyCount", C.c_int32),
                ("awakeCount", C.c_int32), ("contactCount", C.c_int32), ("overflow", C.c_int32),
                ("statesIn", C.c_void_p), ("statesOut", C.c_void_p), ("mass", C.c_void_p),
                ("force", C.c_void_p), ("damping", C.c_void_p), ("awake", C.c_void_p),
                ("contactBodies", C.c_void_p), ("mix", C.c_void_p), ("manifoldsIn", C.c_void_p),
                ("manifoldsOut", C.c_void_p), ("colorStart", C.c_int32 * 13)]


def capture_step(oracle, world, body_cap=20000, contact_cap=60000):
    """Steps `world` once on the oracle; returns the solver stage's inputs and outputs."""
    a = {
        "statesIn": np.zeros((body_cap, 8), np.float32), "statesOut": np.zeros((body_cap, 8), np.float32),
        "mass": np.zeros((body_cap, 4), np.float32), "force": np.zeros((body_cap, 4), np.float32),
        "damping": np.zeros((body_cap, 4), np.float32), "awake": np.zeros(body_cap, np.int32),
        "contactBodies": np.zeros((contact_cap, 2), np.int32), "mix": np.zeros((contact_cap, 2), np.float32),
        "manifoldsIn": np.zeros(contact_cap * MANIFOLD_BYTES, np.uint8),
        "manifoldsOut": np.zeros(contact_cap * MANIFOLD_BYTES, np.uint8),
    }
    cap = Capture(bodyCap=body_cap, contactCap=contact_cap)
    for k, v in a.items():
        setattr(cap, k, v.ctypes.data)
    fn = oracle.lib.b2o_StepCapture
    fn.argtypes = [type(world), C.c_float, C.c_int, C.POINTER(Capture)]
    fn.restype = C.c_int
    assert fn(world, DT, SUBSTEPS, C.byref(cap)) == 0
    nb, na, nc = cap.bodyCount, cap.awakeCount, cap.contactCount
    return {
        "statesIn": a["statesIn"][:nb], "statesOut": a["statesOut"][:nb], "mass": a["mass"][:nb],
        "force": a["force"][:nb], "damping": a["damping"][:nb], "awake": a["awake"][:na],
        "contactBodies": a["contactBodies"][:nc], "mix": a["mix"][:nc],
        "manifoldsIn": a["manifoldsIn"][:nc * MANIFOLD_BYTES], "manifoldsOut": a["manifoldsOut"][:nc * MANIFOLD_BYTES],
        "colorStart": list(cap.colorStart),
    }


def make_desc(torch, cap, dev):
    """Device copies of a capture and the descriptor that points at them."""
    t = {k: torch.from_numpy(np.ascontiguousarray(cap[k])).to(dev)
         for k in ("statesIn", "mass", "force", "damping", "awake", "contactBodies", "mix", "manifoldsIn")}
    d = ContactSolveDesc()
    d.states = t["statesIn"].data_ptr()
    d.massData = t["mass"].data_ptr()
    d.forces = t["force"].data_ptr()
    d.damping = t["damping"].data_ptr()
    d.bodies = t["awake"].data_ptr()
    d.bodyCount = len(cap["awake"])
    d.contactBodies = t["contactBodies"].data_ptr()
    d.contactMix = t["mix"].data_ptr()
    d.manifolds = t["manifoldsIn"].data_ptr()
    d.contactCount = len(cap["contactBodies"])
    for c in range(13):
        d.colorStart[c] = cap["colorStart"][c]
    d.timeStep = DT
    d.subStepCount = SUBSTEPS
    d.gravity = Vec2(0.0, -10.0)
    d.contactHertz = 30.0
    d.contactDampingRatio = 10.0
    d.contactPushout = 3.0
    d.restitutionThreshold = 1.0
    d.enableWarmStarting = True
    d.stream = None
    return d, t


def solve_on_device(gpu, torch, cap):
    bind_solve_api(gpu.lib)
    d, t = make_desc(torch, cap, "cuda:0")
    rc = gpu.lib.b2SolveContacts(C.byref(d))
    torch.cuda.synchronize()
    assert rc == 0
    return t["statesIn"].cpu().numpy(), t["manifoldsIn"].cpu().numpy()


def _scene(oracle, name):
    if name == "pyramid20":
        return oracle.pyramid(20)
    if name == "pyramid_jitter":
        return oracle.pyramid(40, 0.01, 77)
    if name == "tilted":
        return oracle.tilted_stacks()
    raise KeyError(name)


@pytest.mark.gpu
@pytest.mark.parametrize("scene,warm", [("pyramid20", 40), ("pyramid_jitter", 25), ("tilted", 30)])
def test_solve_contacts_matches_oracle_stage(gpu, oracle, scene, warm):
    torch = pytest.importorskip("torch")
    w = _scene(oracle, scene)
    oracle.step(w, DT, SUBSTEPS, warm)
    cap = capture_step(oracle, w)
    oracle.destroy(w)
    assert len(cap["contactBodies"]) > 0
    states, manifolds = solve_on_device(gpu, torch, cap)
    assert np.array_equal(states.view(np.uint32), cap["statesOut"].view(np.uint32))
    assert np.array_equal(manifolds, cap["manifoldsOut"])


@pytest.mark.gpu
def test_solve_contacts_rejects_bad_plan(gpu):
    bind_solve_api(gpu.lib)
    d = ContactSolveDesc()
    assert gpu.lib.b2SolveContacts(C.byref(d)) == -1
    assert gpu.lib.b2SolveContacts(None) == -1
