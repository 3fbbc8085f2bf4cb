"""b2World_StepBatch (include/box2d/gpu.h): many worlds stepped together must give each
world exactly the bits the oracle gives it stepped alone (reference b2World_Step)."""
import ctypes as C

import numpy as np
import pytest

from box2c_gb300.capi import bind_batch_api, contact_table, world_array

pytestmark = pytest.mark.gpu


def _scenes(backend, bases):
    worlds = [backend.pyramid(int(b), 0.01, 100 + i) for i, b in enumerate(bases)]
    worlds.append(backend.tumbler(300, 7, 0))
    worlds.append(backend.hello_world()[0])
    return worlds


def _compare(gpu, oracle, wg, wo):
    for i, (a, b) in enumerate(zip(wg, wo)):
        ta, tb = contact_table(gpu.contacts(a)), contact_table(oracle.contacts(b))
        if ta.shape != tb.shape or not np.array_equal(ta, tb):
            return f"world {i}: contacts/colours differ"
        ba, bb = gpu.bodies(a), oracle.bodies(b)
        if not np.array_equal(ba.view(np.uint32), bb.view(np.uint32)):
            return f"world {i}: body state differs"
    return None


def test_batch_matches_oracle_worlds(gpu, oracle):
    bind_batch_api(gpu.lib)
    rng = np.random.default_rng(5)
    bases = rng.integers(4, 41, size=14)
    wg, wo = _scenes(gpu, bases), _scenes(oracle, bases)
    ids = world_array(wg)
    try:
        for s in range(1, 61):
            gpu.lib.b2World_StepBatch(ids, len(wg), 1.0 / 60.0, 4)
            for w in wo:
                oracle.step(w)
            if s in (1, 2, 5, 10, 30, 60):
                err = _compare(gpu, oracle, wg, wo)
                assert err is None, f"step {s}: {err}"
        stats = gpu.lib.b2World_GetBatchStats()
        assert stats.solveThreads in (64, 128, 256, 512)  # the autotuner has chosen
        assert stats.launches == 4  # scatter, narrowphase, tape records, solver
    finally:
        for w in wg:
            gpu.destroy(w)
        for w in wo:
            oracle.destroy(w)


def test_batch_skips_invalid_and_repeated_ids(gpu, oracle):
    bind_batch_api(gpu.lib)
    a, b = gpu.pyramid(6), oracle.pyramid(6)
    bad = type(a)(index1=4000, revision=1)
    ids = world_array([a, bad, a])
    try:
        for _ in range(20):
            gpu.lib.b2World_StepBatch(ids, 3, 1.0 / 60.0, 4)
            oracle.step(b)
        assert _compare(gpu, oracle, [a], [b]) is None
    finally:
        gpu.destroy(a)
        oracle.destroy(b)


def test_batch_then_single_steps_continue_bit_exact(gpu, oracle):
    """Batched and single steps can be mixed on the same world."""
    bind_batch_api(gpu.lib)
    wg, wo = [gpu.pyramid(12), gpu.pyramid(7)], [oracle.pyramid(12), oracle.pyramid(7)]
    ids = world_array(wg)
    try:
        for s in range(40):
            if s % 3 == 0:
                for w in wg:
                    gpu.step(w)
            else:
                gpu.lib.b2World_StepBatch(ids, 2, 1.0 / 60.0, 4)
            for w in wo:
                oracle.step(w)
        assert _compare(gpu, oracle, wg, wo) is None
    finally:
        for w in wg + wo[:0]:
            gpu.destroy(w)
        for w in wo:
            oracle.destroy(w)


def test_batch_steps_worlds_too_large_for_it_alone(gpu):
    """A world with more bodies than the batched solver holds in shared memory is stepped
    by the single-world path inside the same call; the others are batched."""
    bind_batch_api(gpu.lib)
    make = [lambda: gpu.pyramid(120), lambda: gpu.pyramid(9), lambda: gpu.pyramid(14)]
    wb = [m() for m in make]
    ws = [m() for m in make]
    ids = world_array(wb)
    try:
        for _ in range(4):
            gpu.lib.b2World_StepBatch(ids, len(wb), 1.0 / 60.0, 4)
            for w in ws:
                gpu.step(w)
        for i, (a, b) in enumerate(zip(wb, ws)):
            assert gpu.lib.b2World_GetStatus(a) == 0
            ba, bb = gpu.bodies(a), gpu.bodies(b)
            assert np.array_equal(ba.view(np.uint32), bb.view(np.uint32)), f"world {i}"
    finally:
        for w in wb + ws:
            gpu.destroy(w)


def test_batch_in_halves_matches_single_steps(gpu):
    """Batches with at least 100k bodies run in two halves whose host and device work
    overlap; each world still gets the bits of its own b2World_Step (which the oracle
    tests pin)."""
    bind_batch_api(gpu.lib)
    rng = np.random.default_rng(9)
    bases = rng.integers(30, 41, size=180)
    assert sum(int(b) * (int(b) + 1) // 2 for b in bases) >= 100000
    wb = [gpu.pyramid(int(b), 0.01, 300 + i) for i, b in enumerate(bases)]
    ws = [gpu.pyramid(int(b), 0.01, 300 + i) for i, b in enumerate(bases)]
    ids = world_array(wb)
    try:
        for _ in range(6):
            gpu.lib.b2World_StepBatch(ids, len(wb), 1.0 / 60.0, 4)
            for w in ws:
                gpu.step(w)
        for i, (a, b) in enumerate(zip(wb, ws)):
            ba, bb = gpu.bodies(a), gpu.bodies(b)
            assert np.array_equal(ba.view(np.uint32), bb.view(np.uint32)), f"world {i}"
    finally:
        for w in wb + ws:
            gpu.destroy(w)


def test_batch_full_size_workload(gpu, oracle):
    """The batched workload at full size: 4096 pyramids with bases U{4..40} (the bench's
    seeded draw), 30 batched steps.  Every world ends bit-identical to the same world
    stepped alone with b2World_Step (checked in chunks of 512 worlds), and a sample of 128
    worlds (every 32nd) equals the oracle stepping it."""
    bind_batch_api(gpu.lib)
    steps = 30
    bases = np.random.default_rng(1237).integers(4, 41, size=4096)
    wb = [gpu.pyramid(int(b), 0.0, 0) for b in bases]
    ids = world_array(wb)
    try:
        for _ in range(steps):
            gpu.lib.b2World_StepBatch(ids, len(wb), 1.0 / 60.0, 4)
        assert all(gpu.lib.b2World_GetStatus(w) == 0 for w in wb)
        batched = [gpu.bodies(w) for w in wb]
        tables = [contact_table(gpu.contacts(w)) for w in wb]
    finally:
        for w in wb:
            gpu.destroy(w)
    for start in range(0, len(bases), 512):
        chunk = bases[start:start + 512]
        ws = [gpu.pyramid(int(b), 0.0, 0) for b in chunk]
        try:
            for w in ws:
                gpu.step(w, count=steps)
            for k, w in enumerate(ws):
                i = start + k
                assert np.array_equal(gpu.bodies(w).view(np.uint32), batched[i].view(np.uint32)), f"world {i}"
                assert np.array_equal(contact_table(gpu.contacts(w)), tables[i]), f"world {i} contacts"
        finally:
            for w in ws:
                gpu.destroy(w)
    for i in range(0, len(bases), 32):
        wo = oracle.pyramid(int(bases[i]), 0.0, 0)
        oracle.step(wo, count=steps)
        same = np.array_equal(oracle.bodies(wo).view(np.uint32), batched[i].view(np.uint32))
        oracle.destroy(wo)
        assert same, f"world {i} differs from the oracle"


def test_batch_mixed_paths_match_oracle(gpu, oracle):
    """Batched worlds that take the paths the pyramids do not: capsule and segment
    manifolds, joints in colours and in the overflow colour, motors, and time-of-impact
    events of fast bodies and bullets (handled per world after the batched solver)."""
    bind_batch_api(gpu.lib)
    makers = [lambda b: b.shape_pile(200, 31), lambda b: b.joint_hub(16, 3, 4, 32), lambda b: b.fast_shots(30, 33),
              lambda b: b.many_pyramids(2, 2, 8), lambda b: b.joint_grid(12, -10.0), lambda b: b.pyramid(10)]
    wg = [m(gpu) for m in makers]
    wo = [m(oracle) for m in makers]
    ids = world_array(wg)
    try:
        for s in range(1, 121):
            gpu.lib.b2World_StepBatch(ids, len(wg), 1.0 / 60.0, 4)
            for w in wo:
                oracle.step(w)
            if s % 20 == 0:
                err = _compare(gpu, oracle, wg, wo)
                assert err is None, f"step {s}: {err}"
    finally:
        for w in wg:
            gpu.destroy(w)
        for w in wo:
            oracle.destroy(w)


def test_batch_joint_types_match_oracle(gpu, oracle_atan):
    """Batched worlds with every joint type (the joint scene at two sizes and seeds, next
    to a pyramid and a chain scene): each world bit-identical to the oracle build with the
    library's own atan2, stepped alone."""
    bind_batch_api(gpu.lib)
    makers = [lambda b: b.joint_zoo(1, 0, 61), lambda b: b.joint_zoo(2, 1, 62), lambda b: b.pyramid(12),
              lambda b: b.joint_zoo(1, 1, 63), lambda b: b.chain_scene(120, 64)]
    wg = [m(gpu) for m in makers]
    wo = [m(oracle_atan) for m in makers]
    ids = world_array(wg)
    try:
        for s in range(1, 151):
            gpu.lib.b2World_StepBatch(ids, len(wg), 1.0 / 60.0, 4)
            for w in wo:
                oracle_atan.step(w)
            if s % 10 == 0:
                err = _compare(gpu, oracle_atan, wg, wo)
                assert err is None, f"step {s}: {err}"
    finally:
        for w in wg:
            gpu.destroy(w)
        for w in wo:
            oracle_atan.destroy(w)
