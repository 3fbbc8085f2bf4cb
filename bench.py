"""Benchmark of the per-step contact pipeline on one GB300.

Workload (default): the large pyramid -- 100 rows, 5050 unit boxes with U(-0.01, 0.01) m
x jitter (seed 1235) on a 200 m static ground, dt 1/60, 4 substeps -- stepped with
b2World_Step.  One "step" is one b2World_Step of that world.

Printed JSON line (rank 0):
  value       device-timed ms/step (CUDA events on the world's stream around each step;
              L2 flushed between timed steps, outside the events)
  e2e         ms/step through the C API with host buffers: b2World_Step followed by
              b2World_GetBodyStates (device -> host copy of every body's state)
  roofline    algorithmic bytes of the colour-phase solver stage (per-unit byte model of
              the step path, counted from the live contact and body counts) over its
              device time, against the measured HBM copy bandwidth
  cpu_baseline  the plain-C CPU restatement of the same step on all host cores, over a
              bounded sample of the same step window
  window      the timed steps (W+1 .. W+K after W warm-up steps) and, beside them, the
              same number of steps once the pyramid has settled (from step 100 on)

--impl reference times the CPU implementation of the step (the plain-C restatement
built from oracle/, on all host cores) over the same workload, warm-up and step window
and prints the same metric.
--gpus N: the path does not shard (colour phases are global Gauss-Seidel sweeps), so N
ranks step N independent replicas; value is the slowest rank's ms/step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

METRIC = "ms/step large pyramid; batched world-steps/s; fwd+bwd vs fwd ms, 1 GB300"
BASE = 100
JITTER = 0.01
SEED = 1235
DT = 1.0 / 60.0
SUBSTEPS = 4


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_max(value, dist=None):
    """The maximum of a per-rank figure over all ranks (replicas: each rank steps its own
    world, so the job's time per step is the slowest rank's)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peak():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(contacts, awake_bodies, shape_vertex_counts, substeps):
    """Per-step byte model of the step path (reads + writes each stage must move once).

    contacts: list of point counts of coloured (touching) contacts; the narrowphase also
    visits non-touching contacts (0 points).  Returns (total, solver_stage) in bytes.
    """
    P = np.asarray(contacts["points"], np.int64)
    Pall = np.asarray(contacts["all_points"], np.int64)
    S = substeps
    N = awake_bodies
    collide = int(np.sum(244 + 56 * Pall))
    prepare = int(np.sum(120 + 72 * P))
    intvel = S * N * 60
    warm = S * int(np.sum(80 + 24 * P))
    solve = S * int(np.sum(128 + 52 * P))
    intpos = S * N * 44
    relax = S * int(np.sum(116 + 52 * P))
    restitution = int(np.sum(84 + 36 * P))
    store = int(np.sum(32 * P))
    finalize = N * 128 + int(np.sum(8 * np.asarray(shape_vertex_counts) + 32))
    solver = prepare + intvel + warm + solve + intpos + relax + restitution + store
    total = collide + solver + finalize
    return total, solver


def oracle_backend(threads):
    """The plain-C CPU restatement, its parallel loops (colour rows, bodies, narrowphase
    contacts) on `threads` host threads; any count gives the same bits."""
    subprocess.run(["make", "-s", "-j8", "-f", "oracle/Makefile"], cwd=REPO, check=True, capture_output=True)
    from box2c_gb300.capi import Backend
    ob = os.path.join(REPO, "oracle", "_build")
    o = Backend(os.path.join(ob, "liboracle.so"), os.path.join(ob, "liboracle_scenes.so"), "oracle")
    o.lib.b2o_SetThreads.argtypes = [C.c_int]
    o.lib.b2o_SetThreads.restype = C.c_int
    o.lib.b2o_SetThreads(threads)
    return o


SETTLE_STEPS = 100  # the large pyramid is at rest from about this step on
HOST_PHASES = ("hostPairQuery", "hostPairRules", "hostContactCreate", "hostEvents", "hostSolveLists", "hostTreeRebuild",
               "hostRecords", "hostContinuous")
CPU_SAMPLE_STEPS = 40  # bounded sample of the CPU baseline leg of the GPU arm


def workload_config(world_size=1):
    """The workload both arms name in `config` (identical dicts)."""
    return {"workload": "large_pyramid_100_rows_5050_boxes", "rows": BASE, "bodies": BASE * (BASE + 1) // 2,
            "jitter": JITTER, "seed": SEED, "dt": DT, "substeps": SUBSTEPS, "parallelism": f"replicas{world_size}"}


def oracle_windows(warmup, steps, settled=True, sample=None):
    """The plain-C CPU restatement stepping the large pyramid on all host cores: `warmup`
    untimed steps, then the timed window of `steps` steps (at most `sample` of them), then
    (optionally) the same number of steps once the pyramid has settled.
    Returns (ms/step of the window, steps timed, ms/step settled or None, threads)."""
    cores = os.cpu_count() or 1
    o = oracle_backend(cores)
    w = o.pyramid(BASE, JITTER, SEED)
    o.step(w, DT, SUBSTEPS, count=warmup)
    n = steps if sample is None else min(steps, sample)
    t0 = time.perf_counter()
    o.step(w, DT, SUBSTEPS, count=n)
    ms = (time.perf_counter() - t0) * 1e3 / n
    settled_ms = None
    if settled:
        done = warmup + n
        o.step(w, DT, SUBSTEPS, count=max(0, SETTLE_STEPS - done))
        t0 = time.perf_counter()
        o.step(w, DT, SUBSTEPS, count=n)
        settled_ms = (time.perf_counter() - t0) * 1e3 / n
    o.destroy(w)
    return ms, n, settled_ms, cores


def cpu_baseline(warmup, steps):
    """The CPU baseline beside the GPU arm: the oracle over the GPU arm's timed step window
    (a bounded sample of it), on all host cores."""
    ms, n, _, cores = oracle_windows(warmup, steps, settled=False, sample=CPU_SAMPLE_STEPS)
    return {"value": round(ms, 4), "unit": "ms/step", "cores": cores, "kind": "port",
            "sample": f"steps {warmup + 1}-{warmup + n} of the same 100-row pyramid (the GPU arm's timed window)"}


TUMBLER_BODIES = 2000
OVERFLOW_COLOR = 11  # slot of the overflow colour in b2Counters.colorCounts
TUMBLER_SEED = 1236


def run_tumbler(g, steps=1000, cpu=True):
    """Tumbler: a 20 m hollow box of four walls on a revolute motor (0.05 pi rad/s) with
    2000 boxes (half-extent 0.125) and circles (radius 0.125) at seeded random positions,
    4 substeps, 1000 steps; device and wall ms per b2World_Step, host pair time, and the
    oracle on a bounded sample of the same scene (all host cores)."""
    from box2c_gb300.capi import bind_gpu_api
    L = g.lib
    bind_gpu_api(L)
    w = g.tumbler(TUMBLER_BODIES, TUMBLER_SEED, 0)
    L.b2World_EnableDeviceTiming(w, True)
    wall, dev, solve, pairs = [], [], [], []
    for _ in range(steps):
        t = time.perf_counter()
        L.b2World_Step(w, DT, SUBSTEPS)
        wall.append(time.perf_counter() - t)
        d = L.b2World_GetDeviceTimes(w)
        dev.append(d.step)
        solve.append(d.solve)
        pairs.append(L.b2World_GetProfile(w).pairs)
    status = L.b2World_GetStatus(w)
    counters = g.counters(w)
    g.destroy(w)
    skip = min(50, steps // 2)
    out = {"workload": "tumbler_2000_bodies_revolute_motor", "steps": steps,
           "wall_ms_per_step": round(float(np.mean(wall[skip:])) * 1e3, 4),
           "device_ms_per_step": round(float(np.mean(dev[skip:])), 4),
           "solve_ms": round(float(np.mean(solve[skip:])), 4),
           "host_pairs_ms": round(float(np.mean(pairs[skip:])), 4),
           "overflow_constraints": int(counters.colorCounts[OVERFLOW_COLOR]), "status": status}
    if cpu:
        cores = os.cpu_count() or 1
        o = oracle_backend(cores)
        wo = o.tumbler(TUMBLER_BODIES, TUMBLER_SEED, 0)
        o.step(wo, DT, SUBSTEPS, count=100)
        n = 20
        t0 = time.perf_counter()
        o.step(wo, DT, SUBSTEPS, count=n)
        out["cpu_baseline"] = {"value": round((time.perf_counter() - t0) * 1e3 / n, 4), "unit": "ms/step",
                               "cores": cores, "kind": "port", "sample": f"steps 100-{100 + n} of the same tumbler"}
        o.destroy(wo)
    return out


BATCH_WORLDS = 4096
# DRAM bytes of the solver stage of one large-pyramid step (k_fused_stage 2.35 MB +
# k_solve_fused 2.76 MB), from the committed ncu capture of the same workload
SOLVER_DRAM_BYTES = 5.10e6
# DRAM bytes of the batched solver over 2048 of the batched worlds (both halves), from the
# committed ncu capture of that workload
BATCH_SOLVE_DRAM_BYTES = 3.33e9
BATCH_SEED = 1237


def batch_bases(n=BATCH_WORLDS):
    """Pyramid bases U{4..40} for the batched workload (4096 worlds)."""
    rng = np.random.default_rng(BATCH_SEED)
    return rng.integers(4, 41, size=n)


def run_batch(g, steps, warmup, n_worlds=BATCH_WORLDS):
    """Batched worlds: 4096 pyramids with bases U{4..40} (config-0 material, dt, substeps)
    stepped together with b2World_StepBatch; also times a loop of single-world
    b2World_Step calls over a sample of the same worlds."""
    from box2c_gb300.capi import bind_batch_api, world_array
    import torch
    L = g.lib
    bind_batch_api(L)
    bases = batch_bases(n_worlds)
    worlds = [g.pyramid(int(b), 0.0, 0) for b in bases]
    ids = world_array(worlds)
    n = len(worlds)
    # warm up past the solver autotuner (it times each launch shape on the first steps)
    warm = 0
    while warm < max(3, warmup) or (L.b2World_GetBatchStats().solveThreads == 0 and warm < 100):
        L.b2World_StepBatch(ids, n, DT, SUBSTEPS)
        warm += 1
    torch.cuda.synchronize()
    host, dev_c, dev_s = [], [], []
    prof = []
    t0 = time.perf_counter()
    for _ in range(steps):
        t = time.perf_counter()
        L.b2World_StepBatch(ids, n, DT, SUBSTEPS)
        host.append(time.perf_counter() - t)
        st = L.b2World_GetBatchStats()
        dev_c.append(st.collide)
        dev_s.append(st.solve)
        prof.append((st.hostBegin, st.hostCollide, st.hostMiddle, st.hostSolve, st.hostFinish))
    total = time.perf_counter() - t0
    st = L.b2World_GetBatchStats()
    # loop of single-world steps over a sample (the per-world path)
    sample = worlds[:256]
    t = time.perf_counter()
    for w in sample:
        L.b2World_Step(w, DT, SUBSTEPS)
    loop = len(sample) / (time.perf_counter() - t)
    bodies = int(sum(int(b) * (int(b) + 1) // 2 for b in bases))
    failed = sum(1 for w in worlds if L.b2World_GetStatus(w) != 0)
    # algorithmic bytes of one batched solver launch (solver stage + finalisation of every
    # world, the per-unit model of algorithmic_bytes) from each world's touching contacts
    solve_bytes = 0
    for w, b in zip(worlds, bases):
        c = g.contacts(w)
        t = c[c["colorIndex"] >= 0]
        nb = int(b) * (int(b) + 1) // 2
        _, solver = algorithmic_bytes({"points": t["pointCount"], "all_points": c["pointCount"]}, nb, [4] * nb, SUBSTEPS)
        solve_bytes += solver + nb * 128 + nb * (8 * 4 + 32)
    for w in worlds:
        g.destroy(w)
    value = n * steps / total
    solve_dev = float(np.mean(dev_s))
    peak, peak_kind = measured_peak()
    achieved = solve_bytes / (solve_dev * 1e-3) / 1e9 if solve_dev > 0 else 0.0
    return {
        "metric": "batched world-steps/s", "value": round(value, 1), "unit": "world-steps/s",
        "worlds": n, "bodies": bodies, "steps": steps, "warmup": warm,
        "ms_per_batched_step": round(total * 1e3 / steps, 4),
        "device_ms": {"collide": round(float(np.mean(dev_c)), 4), "solve": round(float(np.mean(dev_s)), 4)},
        "host_ms": dict(zip(("prepare_first_half", "launch_prepare_rebuild", "narrowphase_wait_events_lists",
                             "solver_wait_records", "end_of_step"),
                            [round(float(x), 4) for x in np.mean(np.array(prof), 0)])),
        "host_threads": st.hostThreads, "solve_cta_threads": st.solveThreads, "solve_ctas_per_sm": st.solveCtasPerSm,
        "gpu_launches_per_step": st.launches,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": BATCH_SOLVE_DRAM_BYTES * n / 2048,
                     "traffic_source": "ncu dram__bytes_read+write of k_batch_solve, 2048 worlds (a capture "
                                       "before the per-group descriptor copy) scaled to the worlds stepped "
                                       "(profiles/batch_solver_4096_worlds.txt)",
                     "kernel": "k_batch_solve (solver stage + finalisation, both halves)",
                     "algorithmic_bytes_per_step": int(solve_bytes), "peak_kind": peak_kind},
        "loop_world_steps_per_s": round(loop, 1), "speedup_vs_loop": round(value / loop, 1),
        "failed_worlds": failed,
    }


def fd64_gradient_check(heights, v0, mu, grads, steps=120, sample=16):
    """The gradient against central finite differences of the FP64 CPU restatement of the
    same step (the oracle's double build), per world of a fixed sample: relative error
    |g - fd| / |fd| at eps 1e-3 (the specified step) and at eps 1e-6, and whether the
    finite difference is stable.  All worlds of
    the sample are reported; none is dropped.  Stable: eps 1e-5, 1e-6 and 1e-7 agree
    within 1e-4 relative.  `steps` is the horizon (the workload's 120, or a shorter one
    on which the loss is smooth)."""
    subprocess.run(["make", "-s", "-j8", "-f", "oracle/Makefile"], cwd=REPO, check=True, capture_output=True)
    from box2c_gb300.capi import Backend, WorldId
    ob = os.path.join(REPO, "oracle", "_build")
    o = Backend(os.path.join(ob, "liboracle64.so"), os.path.join(ob, "liboracle64_scenes.so"), "oracle64")
    L = o.lib
    L.b2o_GetBodyStateF64.argtypes = [WorldId, C.c_void_p, C.c_int]
    L.b2o_SetBodyVelocityF64.argtypes = [WorldId, C.c_int, C.c_double, C.c_double, C.c_double]
    L.b2o_SetShapeFrictionF64.argtypes = [WorldId, C.c_int, C.c_double]

    def loss(h, v, m):
        w = o.drop_boxes(h, v[:, 0].astype(np.float32), v[:, 1].astype(np.float32), float(m))
        for k in range(len(h)):
            L.b2o_SetBodyVelocityF64(w, k + 1, float(v[k, 0]), float(v[k, 1]), 0.0)
        for sh in range(len(h) + 1):
            L.b2o_SetShapeFrictionF64(w, sh, float(m))
        o.step(w, DT, SUBSTEPS, count=steps)
        st = np.zeros(7 * (len(h) + 1))
        L.b2o_GetBodyStateF64(w, st.ctypes.data, len(h) + 1)
        o.destroy(w)
        return float((st.reshape(-1, 7)[1:, :2] ** 2).sum())

    def fd(h, v, m, eps):
        v = v.astype(np.float64)
        out = np.zeros(v.size + 1)
        for i in range(v.size):
            vp, vm = v.copy(), v.copy()
            vp.flat[i] += eps
            vm.flat[i] -= eps
            out[i] = (loss(h, vp, m) - loss(h, vm, m)) / (2 * eps)
        out[-1] = (loss(h, v, float(m) + eps) - loss(h, v, float(m) - eps)) / (2 * eps)
        return out

    rows = []
    for w in range(sample):
        g = grads[w]
        f3, f5, f6, f7 = (fd(heights[w], v0[w], mu[w], e) for e in (1e-3, 1e-5, 1e-6, 1e-7))
        n6 = np.linalg.norm(f6)
        stable = bool(np.linalg.norm(f5 - f6) <= 1e-4 * n6 and np.linalg.norm(f7 - f6) <= 1e-4 * n6)
        rows.append((float(np.linalg.norm(g - f3) / np.linalg.norm(f3)), float(np.linalg.norm(g - f6) / np.linalg.norm(f6)),
                     stable))
    e3 = np.array([r[0] for r in rows])
    e6 = np.array([r[1] for r in rows])
    st = np.array([r[2] for r in rows])

    def summary(x):
        return {"median": float(np.median(x)), "max": float(np.max(x)),
                "within_1e-3": int(np.sum(x <= 1e-3))} if len(x) else None

    return {"sample": f"worlds 0-{sample - 1} of the 256, {steps} steps, loss sum |p|^2, 17 parameters per world",
            "eps_1e-3": summary(e3), "eps_1e-6": summary(e6), "stable_fraction": float(np.mean(st)),
            "stable_eps_1e-6": summary(e6[st]), "per_world_eps_1e-3": [round(float(x), 6) for x in e3],
            "per_world_eps_1e-6": [round(float(x), 6) for x in e6], "per_world_stable": [bool(x) for x in st]}


def run_adjoint(g, reps=3, check=True):
    """Differentiable stepping: 256 worlds x 8 boxes (half-extent 0.5) dropped from
    U(1,5) m with N(0,1) velocities and per-world friction U(0.2,0.9), 120 steps x 4
    substeps; loss = sum of squared final positions; gradient w.r.t. initial velocities
    and friction by b2World_StepBackwardBatch.  Times the stepped forward (plain and
    recording) and the backward pass."""
    import torch
    from box2c_gb300.autograd import DropBoxes
    rng = np.random.default_rng(1238)
    n = 256
    heights = rng.uniform(1, 5, size=(n, 8)).astype(np.float32)
    v0 = rng.normal(0, 1, size=(n, 8, 2)).astype(np.float32)
    mu = rng.uniform(0.2, 0.9, size=n).astype(np.float32)
    sim = DropBoxes(g, heights, steps=120, substeps=SUBSTEPS, dt=DT)
    plain, taped, back = [], [], []
    for r in range(reps + 1):
        sim.create(v0, mu, record=False)
        torch.cuda.synchronize()
        t = time.perf_counter()
        sim.step_all()
        p0 = sim.positions()
        plain.append(time.perf_counter() - t)
        sim.create(v0, mu, record=True)
        torch.cuda.synchronize()
        t = time.perf_counter()
        sim.step_all()
        p = sim.positions()
        taped.append(time.perf_counter() - t)
        t = time.perf_counter()
        gv, gm = sim.backward(2.0 * p)
        back.append(time.perf_counter() - t)
    sim.destroy()
    f0, f1, bw = (1e3 * float(np.median(x[1:])) for x in (plain, taped, back))
    grads = np.concatenate([gv.reshape(n, -1), gm[:, None]], axis=1)
    check_out = None
    if check:
        check_out = {"steps_120": fd64_gradient_check(heights, v0, mu, grads)}
        # the same worlds over a horizon on which the boxes have not yet collided with
        # each other and tipped: the loss is smooth there
        short = DropBoxes(g, heights[:16], steps=30, substeps=SUBSTEPS, dt=DT)
        p30 = short.run(v0[:16], mu[:16])
        gv30, gm30 = short.backward(2.0 * p30)
        short.destroy()
        g30 = np.concatenate([gv30.reshape(16, -1), gm30[:, None]], axis=1)
        check_out["steps_30"] = fd64_gradient_check(heights[:16], v0[:16], mu[:16], g30, steps=30)
    return {
        "metric": "fwd+bwd vs fwd ms", "workload": "256 worlds x 8 boxes, 120 steps x 4 substeps",
        "fwd_ms": round(f0, 3), "fwd_recording_ms": round(f1, 3), "bwd_ms": round(bw, 3),
        "fwd_plus_bwd_ms": round(f1 + bw, 3), "ratio_vs_fwd": round((f1 + bw) / f0, 3),
        "same_final_state": bool(np.array_equal(p0, p)), "grad_norm": float(np.linalg.norm(gv)),
        "status": sim.last_status, "grad_rel_err": check_out,
    }


def batch_cpu_baseline(sample=1024, steps=5):
    """The plain-C CPU restatement stepping a sample of the batched worlds, one world per
    task on all host cores (worlds are independent)."""
    from concurrent.futures import ThreadPoolExecutor
    o = oracle_backend(1)  # the worlds run in parallel, each on one thread
    worlds = [o.pyramid(int(b), 0.0, 0) for b in batch_bases()[:sample]]
    cores = os.cpu_count() or 1
    with ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(lambda w: o.step(w, DT, SUBSTEPS, count=2), worlds))
        t0 = time.perf_counter()
        list(ex.map(lambda w: o.step(w, DT, SUBSTEPS, count=steps), worlds))
        dt = time.perf_counter() - t0
    for w in worlds:
        o.destroy(w)
    return {"value": round(len(worlds) * steps / dt, 1), "unit": "world-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(worlds)} of the 4096 worlds x {steps} steps after 2 warm-up steps, one world per task"}


def run_reference(args):
    """Reference arm: the CPU implementation of the step on the machine's host cores, over the
    same workload, warm-up and timed steps as the GPU arm (steps W+1 .. W+K of the large
    pyramid), with the settled window reported beside it."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    warm = max(3, args.warmup)
    ms, n, settled_ms, cores = oracle_windows(warm, args.steps)
    line = {"metric": METRIC, "value": round(ms, 4), "unit": "ms/step", "n_gpus": args.gpus, "steps": n,
            "warmup": warm, "ms_per_step": round(ms, 4), "higher_is_better": False, "impl": "reference",
            "dtype": "f32", "data": "synthetic", "scaling": "weak", "vs_baseline": None,
            "config": workload_config(args.gpus),
            "window": {"timed_steps": [warm + 1, warm + n],
                       "settled_steps": [max(SETTLE_STEPS, warm + n) + 1, max(SETTLE_STEPS, warm + n) + n],
                       "settled_ms_per_step": round(settled_ms, 4)},
            "cpu_baseline": {"value": round(ms, 4), "unit": "ms/step", "cores": cores, "kind": "port",
                             "sample": f"steps {warm + 1}-{warm + n} of the 100-row pyramid (the GPU arm's window), "
                                       "the oracle on every host core"},
            "e2e": {"value": round(ms, 4), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_gpu(args):
    import box2c_gb300
    from box2c_gb300.capi import bind_gpu_api

    rank, world_size, local = dist_env()
    if world_size > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    dist = None
    if world_size > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")

    import torch
    box2c_gb300.build()
    g = box2c_gb300.load()
    L = g.lib
    bind_gpu_api(L)

    warm = max(3, args.warmup)
    w = g.pyramid(BASE, JITTER, SEED)
    L.b2World_EnableDeviceTiming(w, True)
    for _ in range(warm):
        g.step(w, DT, SUBSTEPS)

    # L2 is flushed between timed steps by writing a buffer larger than the 129 MB L2
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def device_window(count):
        rec = {"step": [], "solve": [], "collide": [], "finalize": [], "launches": [], "fused": 0, "host": [],
               "phases": []}
        for _ in range(count):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            g.step(w, DT, SUBSTEPS)
            t = L.b2World_GetDeviceTimes(w)
            rec["step"].append(t.step)
            rec["solve"].append(t.solve)
            rec["collide"].append(t.collide)
            rec["finalize"].append(t.finalize)
            rec["launches"].append(t.launches)
            rec["fused"] += t.fusedSolver
            rec["phases"].append([getattr(t, f) for f in HOST_PHASES])
            p = L.b2World_GetProfile(w)
            rec["host"].append((p.step, p.pairs, p.collide, p.solve, p.broadphase))
        return rec

    # timed window: steps warm+1 .. warm+K of the pyramid (the reference arm times the
    # same steps of the same scene)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    with sampler:
        rec = device_window(args.steps)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = replica_max(float(np.mean(rec["step"])), dist)
    solve_ms, collide_ms, finalize_ms = rec["solve"], rec["collide"], rec["finalize"]

    # settled window: the same number of steps once the pyramid has come to rest
    # (from step SETTLE_STEPS on), reported beside the timed window
    done = warm + args.steps
    for _ in range(max(0, SETTLE_STEPS - done)):
        g.step(w, DT, SUBSTEPS)
    settled = device_window(args.steps)
    settled_ms = float(np.mean(settled["step"]))

    contacts = g.contacts(w)
    touching = contacts[contacts["colorIndex"] >= 0]
    cinfo = {"points": touching["pointCount"], "all_points": contacts["pointCount"]}
    counters = g.counters(w)
    shapes = g.shapes(w)
    n_bodies = L.b2World_GetBodyStates(w, None, 0)
    total_bytes, solver_bytes = algorithmic_bytes(cinfo, n_bodies - 1, [4] * (len(shapes) - 1), SUBSTEPS)
    solve_dev = float(np.mean(solve_ms))
    peak, peak_kind = measured_peak()
    achieved = solver_bytes / (solve_dev * 1e-3) / 1e9 if solve_dev > 0 else 0.0
    status = L.b2World_GetStatus(w)
    toi = L.b2World_GetToiEventCount(w)
    g.destroy(w)

    # end to end through the C API with host buffers, over the same step window of a
    # fresh world: b2World_Step, then every body's state copied to a host array; the
    # library counts the bytes each step moves between host and device
    w = g.pyramid(BASE, JITTER, SEED)
    for _ in range(warm):
        L.b2World_Step(w, DT, SUBSTEPS)
    host = np.zeros(7 * n_bodies, np.float32)
    h2d, d2h = [], []
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.b2World_Step(w, DT, SUBSTEPS)
        L.b2World_GetBodyStates(w, host.ctypes.data, n_bodies)
        t = L.b2World_GetDeviceTimes(w)
        h2d.append(t.hostToDeviceBytes)
        d2h.append(t.deviceToHostBytes)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if dist:
        dist.barrier()
    e2e_ms = replica_max(e2e_ms, dist)
    g.destroy(w)

    batch = run_batch(g, args.batch_steps, 5, args.batch_worlds) if args.batch_steps > 0 else None
    tumbler = run_tumbler(g, steps=args.tumbler_steps, cpu=not args.no_cpu) if not args.no_tumbler else None
    adjoint = run_adjoint(g, check=not args.no_cpu) if not args.no_adjoint else None

    if rank != 0:
        return
    cpu = cpu_baseline(warm, args.steps) if not args.no_cpu else None
    if batch is not None and not args.no_cpu:
        batch["cpu_baseline"] = batch_cpu_baseline()
    clocks = sampler.summary()
    line = {
        "metric": METRIC, "value": round(ms, 4), "unit": "ms/step", "n_gpus": world_size, "steps": args.steps,
        "warmup": warm, "ms_per_step": round(ms, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world_size),
        "window": {"timed_steps": [warm + 1, warm + args.steps],
                   "settled_steps": [max(SETTLE_STEPS, done) + 1, max(SETTLE_STEPS, done) + args.steps],
                   "settled_ms_per_step": round(settled_ms, 4),
                   "settled_solve_ms": round(float(np.mean(settled["solve"])), 4)},
        "scene": {"bodies": n_bodies - 1, "contacts": int(len(contacts)), "touching": int(len(touching)),
                  "colors": list(counters.colorCounts), "l2": "flushed between timed steps (256 MB write)",
                  "solver": "fused cluster kernel" if rec["fused"] == args.steps else "per-phase kernels"},
        "stages_ms": {"collide": round(float(np.mean(collide_ms)), 4), "solve": round(solve_dev, 4),
                      "finalize": round(float(np.mean(finalize_ms)), 4)},
        "host_ms": dict(zip(("step", "pairs", "collide_and_events", "solve_and_sync", "records"),
                            [round(float(x), 4) for x in np.mean(np.array(rec["host"]), 0)])),
        "host_phase_ms": {"timed": dict(zip(HOST_PHASES, [round(float(x), 4) for x in np.mean(np.array(rec["phases"]), 0)])),
                          "settled": dict(zip(HOST_PHASES,
                                              [round(float(x), 4) for x in np.mean(np.array(settled["phases"]), 0)]))},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": SOLVER_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read+write of k_fused_stage + k_solve_fused, one step "
                                       "(profiles/solver_fused_large_pyramid.txt)",
                     "kernel": "solver stage (prepare..store)",
                     "algorithmic_bytes_per_step": solver_bytes, "peak_kind": peak_kind},
        "step_roofline": {"algorithmic_bytes_per_step": total_bytes,
                          "achieved_gbs": round(total_bytes / (ms * 1e-3) / 1e9, 2)},
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/step", "h2d_bytes_per_step": int(np.mean(h2d)),
                "d2h_bytes_per_step": int(np.mean(d2h)),
                "bytes_source": "counted by the library per step (b2DeviceTimes host/device bytes): staged contacts, "
                                "solve lists, counters, mapped events and records, and the body-state download of "
                                "b2World_GetBodyStates"},
        "gpu_launches": int(sum(rec["launches"])),
        "cpu_baseline": cpu,
        "clocks": clocks, "status": status, "toi_events": toi,
        "batched": batch,
        "tumbler": tumbler,
        "differentiable": adjoint,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=30, help="batched-worlds steps to time (0: skip)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-stepping measurement")
    ap.add_argument("--no-tumbler", action="store_true", help="skip the tumbler measurement")
    ap.add_argument("--part", default="all", choices=["all", "batch", "tumbler", "adjoint"],
                    help="one workload only (for profiling), printed as its own line")
    ap.add_argument("--tumbler-steps", type=int, default=1000, help="steps of the tumbler measurement")
    ap.add_argument("--batch-worlds", type=int, default=BATCH_WORLDS, help="worlds of the batched workload")
    args = ap.parse_args()
    if args.part != "all":
        import box2c_gb300
        g = box2c_gb300.load()
        if args.part == "batch":
            out = run_batch(g, args.batch_steps, args.warmup, args.batch_worlds)
        elif args.part == "tumbler":
            out = run_tumbler(g, steps=args.tumbler_steps, cpu=not args.no_cpu)
        else:
            out = run_adjoint(g)
        print(json.dumps(out))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
