"""Step-by-step comparison of two box2d backends on the same seeded scene."""
import numpy as np

from box2c_gb300.capi import contact_table


def state_bits(backend, world):
    b = backend.bodies(world)
    return b, b.view(np.uint32)


def lockstep(a, b, make, steps, dt=1.0 / 60.0, substeps=4, check_manifolds=False, after_step=None,
             check_islands=False):
    """Steps both backends; returns (first mismatching step or None, detail, worst rel err).
    after_step(backend, world, step), when given, runs on both after each step (world
    edits such as destruction); check_islands compares every body's solver set and
    island id."""
    wa, wb = make(a), make(b)
    worst = 0.0
    try:
        for s in range(steps + 1):
            ba, ua = state_bits(a, wa)
            bb, ub = state_bits(b, wb)
            ta, tb = contact_table(a.contacts(wa)), contact_table(b.contacts(wb))
            if ta.shape != tb.shape or not np.array_equal(ta, tb):
                return s, "contact set / colours differ", worst
            if check_islands:
                ia, ib = a.islands(wa), b.islands(wb)
                if ia.shape != ib.shape or not np.array_equal(ia, ib):
                    return s, "solver sets / islands differ", worst
            if not np.array_equal(ua, ub):
                m = np.isfinite(ba) & np.isfinite(bb)
                rel = np.abs(ba[m] - bb[m]) / np.maximum(np.abs(bb[m]), 1.0)
                worst = max(worst, float(rel.max()))
                return s, f"body state differs (max rel {rel.max():.3e})", worst
            if check_manifolds:
                ca, cb = a.contacts(wa), b.contacts(wb)
                for f in ("normal",):
                    if not np.array_equal(ca[f].view(np.uint32), cb[f].view(np.uint32)):
                        return s, "manifold normals differ", worst
                pa, pb = ca["points"], cb["points"]
                for f in ("anchorA", "anchorB", "separation", "normalImpulse", "tangentImpulse"):
                    if not np.array_equal(pa[f].view(np.uint32), pb[f].view(np.uint32)):
                        return s, f"manifold {f} differs", worst
            if s < steps:
                a.step(wa, dt, substeps)
                b.step(wb, dt, substeps)
                if after_step is not None:
                    after_step(a, wa, s + 1)
                    after_step(b, wb, s + 1)
        return None, "bit-exact", worst
    finally:
        a.destroy(wa)
        b.destroy(wb)


def run_world_api_checks(backend):
    """Reference test/test_world.c:121-204 (DestroyAllBodiesWorld, TestIsValid): bodies
    created one per step and then destroyed one per step leave no body behind; ids are
    invalid after destruction and after the world is destroyed."""
    L = backend.lib
    w = backend.scenes.b2s_empty_world()
    assert L.b2World_IsValid(w)
    ids = []
    creating = True
    for _ in range(2 * 10 + 10):
        if creating:
            if len(ids) < 10:
                ids.append(backend.scenes.b2s_add_square(w, 0.5))
            else:
                creating = False
        elif ids:
            L.b2DestroyBody(ids.pop())
        L.b2World_Step(w, 1.0 / 60.0, 3)
    assert backend.counters(w).bodyCount == 0
    L.b2DestroyWorld(w)
    assert not L.b2World_IsValid(w)

    w = backend.scenes.b2s_empty_world()
    b1 = backend.scenes.b2s_add_body(w, 0)
    assert L.b2Body_IsValid(b1)
    b2 = backend.scenes.b2s_add_body(w, 0)
    assert L.b2Body_IsValid(b2)
    L.b2DestroyBody(b1)
    assert not L.b2Body_IsValid(b1)
    L.b2DestroyBody(b2)
    assert not L.b2Body_IsValid(b2)
    L.b2DestroyWorld(w)
    assert not L.b2World_IsValid(w)
    assert not L.b2Body_IsValid(b2) and not L.b2Body_IsValid(b1)
