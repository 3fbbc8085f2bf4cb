"""The host fork-join pool (box2c_gb300/csrc/pool.c) that runs per-world host phases of
batched steps and the pair rules of a single step: compiled with a small C harness and
run on the CPU (tests/c/pool_check.c)."""
import os
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pool_jobs_and_try_lock(tmp_path):
    exe = str(tmp_path / "pool_check")
    src = os.path.join(REPO, "box2c_gb300", "csrc")
    subprocess.run(["gcc", "-std=gnu17", "-O2", "-pthread", "-I", src, "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c", "pool_check.c"), os.path.join(src, "pool.c"), "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
