"""Host modules of the library checked on the CPU with small C harnesses (tests/c/): the
fork-join pool that runs per-world host phases of batched steps and the pair rules of a
single step (pool.c), and the dynamic tree whose traversal order fixes contact ids
(tree.c, against the oracle's tree)."""
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


def test_host_tree_matches_oracle_tree(tmp_path):
    """The library's host dynamic tree against the oracle's under a seeded sequence of
    creates, moves, enlargements, destroys and rebuilds (tests/c/tree_check.c)."""
    exe = str(tmp_path / "tree_check")
    src = os.path.join(REPO, "box2c_gb300", "csrc")
    inc = os.path.join(REPO, "include")
    flags = ["-std=gnu17", "-O2", "-ffp-contract=off", "-I", inc]
    objs = []
    for name, extra, files in (
            ("product", ["-I", src, "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")],
             [os.path.join(REPO, "tests", "c", "tree_product.c"), os.path.join(src, "tree.c"), os.path.join(src, "util.c")]),
            ("oracle", ["-I", os.path.join(REPO, "oracle")],
             [os.path.join(REPO, "tests", "c", "tree_oracle.c"), os.path.join(REPO, "oracle", "b2o_tree.c")])):
        for f in files:
            obj = str(tmp_path / (name + "_" + os.path.basename(f) + ".o"))
            subprocess.run(["gcc", *flags, *extra, "-c", f, "-o", obj], check=True, capture_output=True)
            objs.append(obj)
    subprocess.run(["gcc", os.path.join(REPO, "tests", "c", "tree_check.c"), *objs, "-lm", "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")


def test_batched_world_packing(tmp_path):
    """The batched solver's packing of worlds into CTAs (box2c_gb300/csrc/b2g_packs.h) on
    seeded random batches (tests/c/packs_check.cpp)."""
    exe = str(tmp_path / "packs_check")
    src = os.path.join(REPO, "box2c_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", src, "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c", "packs_check.cpp"), "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")


def test_time_of_impact_matches_oracle(tmp_path):
    """The library's time of impact and GJK distance (box2c_gb300/csrc/b2g_toi.h, host
    build) against the oracle's (oracle/b2o_toi.c) on seeded random proxies and sweeps:
    same time bits, same outcome, same distance bits (tests/c/toi_check.c)."""
    exe = str(tmp_path / "toi_check")
    src = os.path.join(REPO, "box2c_gb300", "csrc")
    inc = os.path.join(REPO, "include")
    flags = ["-std=gnu17", "-O2", "-ffp-contract=off", "-I", inc]
    objs = []
    for name, extra, files in (
            ("product", ["-I", src], [os.path.join(REPO, "tests", "c", "toi_product.c")]),
            ("oracle", ["-I", os.path.join(REPO, "oracle")],
             [os.path.join(REPO, "tests", "c", "toi_oracle.c"), os.path.join(REPO, "oracle", "b2o_toi.c")])):
        for f in files:
            obj = str(tmp_path / (name + "_" + os.path.basename(f) + ".o"))
            subprocess.run(["gcc", *flags, *extra, "-c", f, "-o", obj], check=True, capture_output=True)
            objs.append(obj)
    subprocess.run(["gcc", os.path.join(REPO, "tests", "c", "toi_check.c"), *objs, "-lm", "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout


def test_joint_angle_atan2(tmp_path):
    """The library's atan2 for joint angles (box2c_gb300/csrc/b2g_math.h gatan2) against
    the oracle's copy (bit for bit) and the C library's atan2f (one ulp at most) on
    rotation-like, small-angle, general and signed-zero inputs (tests/c/atan_check.c)."""
    exe = str(tmp_path / "atan_check")
    src = os.path.join(REPO, "box2c_gb300", "csrc")
    flags = ["-std=gnu17", "-O2", "-ffp-contract=off", "-I", os.path.join(REPO, "include")]
    objs = []
    for f, extra in (("atan_product.c", ["-I", src]), ("atan_oracle.c", ["-I", os.path.join(REPO, "oracle")])):
        obj = str(tmp_path / (f + ".o"))
        subprocess.run(["gcc", *flags, *extra, "-c", os.path.join(REPO, "tests", "c", f), "-o", obj],
                       check=True, capture_output=True)
        objs.append(obj)
    subprocess.run(["gcc", *flags, os.path.join(REPO, "tests", "c", "atan_check.c"), *objs, "-lm", "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
