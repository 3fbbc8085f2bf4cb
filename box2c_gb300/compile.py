"""Builds the GB300 step library (C host code + sm_103a CUDA) in-tree.

Outputs into box2c_gb300/_build/:
  libbox2d_gb300.so         the box2d C API backed by the device pipeline
  libbox2d_gb300_scenes.so  the benchmark scene generators linked against it

Flags that matter for results: host C is compiled with -ffp-contract=off and device
code with --fmad=false, so no multiply-add is fused anywhere (the reference's x86 build
has no FMA); division and square root stay IEEE (-prec-div/-prec-sqrt defaults).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(REPO, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels.cu", "fused.cu", "batch.cu", "adjoint.cu", "arena.cu", "pairs.cu", "solve_api.cu", "solve_noalloc.cu"]
C_SOURCES = ["world.c", "joint.c", "island.c", "step.c", "batch.c", "pool.c", "adjoint.c", "tree.c", "util.c", "geometry.c"]
HEADERS = ["b2g_math.h", "b2g_types.h", "b2g_collide.h", "b2g_device.h", "b2g_solve.h", "b2g_joints.h", "b2g_stages.h", "b2g_dual.h", "b2g_cluster.h", "b2g_packs.h", "host.h"]

LIB = os.path.join(OUT, "libbox2d_gb300.so")
SCENES = os.path.join(OUT, "libbox2d_gb300_scenes.so")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _header_deps() -> list[str]:
    hs = [os.path.join(SRC, h) for h in HEADERS]
    hs += [os.path.join(INC, "box2d", f) for f in os.listdir(os.path.join(INC, "box2d"))]
    return hs + [os.path.abspath(__file__)]


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles what changed; returns the path of libbox2d_gb300.so."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}; set CUDA_HOME")
    os.makedirs(OUT, exist_ok=True)
    hdrs = _header_deps()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-I", INC, "-I", SRC, "-c", src, "-o", obj])
    for f in C_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append(["gcc", "-std=gnu17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-strict-aliasing", "-Wall",
                         "-Wno-unused-function", "-I", INC, "-I", SRC, "-I", os.path.join(CUDA_HOME, "include"),
                         "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, exc in zip(jobs, ex.map(lambda c: _try(c, verbose), jobs)):
                if exc is not None:
                    raise exc
    if force or jobs or _newer(LIB, objs):
        _run(["g++", "-shared", "-Wl,-Bsymbolic", "-Wl,-soname,libbox2d_gb300.so", "-o", LIB, *objs,
              "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart_static", "-ldl", "-lpthread", "-lrt"])
    scene_src = os.path.join(SRC, "scenes.c")
    if force or _newer(SCENES, [scene_src, LIB, os.path.join(SRC, "scenes.h")] + hdrs):
        _run(["gcc", "-std=gnu17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INC, "-I", SRC, "-shared",
              "-o", SCENES, scene_src, "-L", OUT, "-lbox2d_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    return LIB


def _try(cmd, verbose):
    try:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            return RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return None
    except Exception as e:  # pragma: no cover - surfaced to the caller
        return e


def clean() -> None:
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
