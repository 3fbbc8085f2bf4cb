"""Generates the golden fixtures in tests/golden/ from the reference build.

Run in a container that has the reference sources (it builds oracle/_ref first):

    python tests/golden/make_golden.py

Fixtures (all produced by the unmodified reference library, oracle/_ref/libb2ref.so):
  scenes.npz     per-step hashes of body state bits, of the contact table (contact id,
                 shape pair, colour, touching, point count) and of every body's solver
                 set and island id, plus full body snapshots, for the scenes of SCENES;
  manifolds.npz  seeded random shape pairs and the reference manifolds for them;
  smooth_manifolds.npz  seeded chain links against every shape type: the reference's
                 manifolds and closest-feature caches from an empty and a warmed cache.
The GPU machine has no reference sources; its tests read these files instead.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from box2c_gb300.capi import Backend, contact_table  # noqa: E402
from tests.golden.shapes import (Manifold, Polygon, Circle, Capsule, Transform,  # noqa: E402
                                 random_pairs, manifold_array, random_smooth_pairs, collide_smooth)

SCENES = {
    # name: (steps, snapshot steps)
    "pyramid20": (300, (1, 10, 60, 150, 300)),
    "tumbler2000": (200, (1, 50, 100, 200)),
    "tilted": (100, (1, 50, 100)),
    # default world def has sleep on: the body's island falls asleep at step 88
    "hello": (200, (87, 88, 200)),
    "pyramid100": (40, (40,)),
    # reference benchmark/joint_grid.c with gravity, at 30 x 30 and at the benchmark's
    # 100 x 100 (19800 revolute joints in the graph colours)
    "joint_grid30": (120, (1, 60, 120)),
    "joint_grid100": (30, (30,)),
    # reference benchmark/many_pyramids.c: 5 x 5 and the benchmark's 20 x 20 pyramids on
    # static segments
    "many_pyramids5": (120, (1, 60, 120)),
    "many_pyramids20": (30, (30,)),
    # capsules, segments, circles, boxes and rounded boxes; time-of-impact events
    "shape_pile": (300, (1, 100, 200, 300)),
    # joints in the overflow colour; with limits, springs and motors (flags 7)
    "joint_hub": (300, (1, 100, 200, 300)),
    "joint_hub_limits": (300, (1, 100, 200, 300)),
    # contact-free revolute chains with limits, springs and motors
    "joint_chains": (300, (1, 2, 10, 60, 300)),
    # projectiles and bullets against a thin wall: continuous collision
    "fast_shots": (200, (1, 50, 100, 200)),
    # every joint type (distance, motor, mouse, prismatic, revolute, weld, wheel), in the
    # graph colours and in the overflow colour, with contacts
    "joint_zoo": (300, (1, 2, 10, 60, 300)),
    "joint_zoo_collide": (200, (1, 2, 10, 100, 200)),
    # chains: smooth segments (terrain and a closed bowl) against every shape type, bullets
    "chain_scene": (300, (1, 10, 60, 150, 300)),
    # islands and sleep: piles and a chain fall asleep, sets merge through a joint, and
    # destruction, contact, velocity and the sleep switches wake them (scripted steps)
    "sleep_scene": (360, (1, 60, 120, 200, 300, 360)),
}

# scenes edited between steps: backend method called with (world, step number)
STEPPERS = {"sleep_scene": "sleep_step"}


def make_scene(b: Backend, name: str):
    if name == "pyramid20":
        return b.pyramid(20)
    if name == "pyramid100":
        return b.pyramid(100, 0.01, 1235)
    if name == "tumbler2000":
        return b.tumbler(2000, 1236, 0)
    if name == "tilted":
        return b.tilted_stacks()
    if name == "hello":
        return b.hello_world()[0]
    if name == "joint_grid30":
        return b.joint_grid(30, -10.0)
    if name == "joint_grid100":
        return b.joint_grid(100, -10.0)
    if name == "many_pyramids5":
        return b.many_pyramids(5, 5, 10)
    if name == "many_pyramids20":
        return b.many_pyramids(20, 20, 10)
    if name == "shape_pile":
        return b.shape_pile(600, 1239)
    if name == "joint_hub":
        return b.joint_hub(20, 6, 0, 1240)
    if name == "joint_hub_limits":
        return b.joint_hub(20, 6, 7, 1240)
    if name == "joint_chains":
        return b.joint_chains(8, 8, 7, 1242)
    if name == "fast_shots":
        return b.fast_shots(60, 1241)
    if name == "joint_zoo":
        return b.joint_zoo(2, 0, 1250)
    if name == "joint_zoo_collide":
        return b.joint_zoo(3, 1, 1251)
    if name == "chain_scene":
        return b.chain_scene(200, 1260)
    if name == "sleep_scene":
        return b.sleep_scene()
    raise KeyError(name)


def step_scene(b: Backend, name: str, w, s: int) -> None:
    """Advances scene `name` from step s-1 to step s (the step, then its scripted edits)."""
    b.step(w)
    if name in STEPPERS:
        getattr(b, STEPPERS[name])(w, s)


def digest(arr: np.ndarray) -> np.uint64:
    h = hashlib.sha256(np.ascontiguousarray(arr).tobytes()).digest()
    return np.frombuffer(h[:8], dtype=np.uint64)[0]


def record(b: Backend, name: str):
    steps, snaps = SCENES[name]
    w = make_scene(b, name)
    body_h, contact_h, island_h, snap = [], [], [], {}
    for s in range(steps + 1):
        bodies = b.bodies(w)
        table = contact_table(b.contacts(w))
        body_h.append(digest(bodies.view(np.uint32)))
        contact_h.append(digest(table))
        island_h.append(digest(b.islands(w)))
        if s in snaps:
            snap[s] = bodies.copy()
        if s < steps:
            step_scene(b, name, w, s + 1)
    b.destroy(w)
    return np.array(body_h, np.uint64), np.array(contact_h, np.uint64), np.array(island_h, np.uint64), snap


def main():
    subprocess.run(["make", "-s", "-j8", "-f", "oracle/Makefile.ref", "REF=/root/reference"], cwd=REPO, check=True)
    ref = Backend(os.path.join(REPO, "oracle/_ref/libb2ref.so"), os.path.join(REPO, "oracle/_ref/libb2ref_scenes.so"), "ref")
    out = {}
    for name in SCENES:
        bh, ch, ih, snap = record(ref, name)
        out[f"{name}/body_hash"] = bh
        out[f"{name}/contact_hash"] = ch
        out[f"{name}/island_hash"] = ih
        for s, arr in snap.items():
            out[f"{name}/bodies_{s}"] = arr
    np.savez_compressed(os.path.join(HERE, "scenes.npz"), **out)

    pairs = random_pairs(seed=7, count=400)
    L = ref.lib
    results = []
    for kind, a, xa, b, xb in pairs:
        fn = getattr(L, kind)
        fn.restype = Manifold
        fn.argtypes = [C.c_void_p, Transform, C.c_void_p, Transform]
        m = fn(C.addressof(a), xa, C.addressof(b), xb)
        results.append(manifold_array(m))
    np.savez_compressed(os.path.join(HERE, "manifolds.npz"), outputs=np.stack(results))
    smooth = [collide_smooth(L, e) for e in random_smooth_pairs(seed=11, count=400)]
    np.savez_compressed(os.path.join(HERE, "smooth_manifolds.npz"), outputs=np.stack(smooth))
    print("wrote", os.path.join(HERE, "scenes.npz"), "manifolds.npz and smooth_manifolds.npz")


if __name__ == "__main__":
    main()
