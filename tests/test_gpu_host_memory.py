"""Host memory through the reference's allocator hook (b2SetAllocator / b2GetByteCount,
reference src/allocate.c:39-107), with failures injected by the hook.

tests/c/alloc_fault.c installs an allocator that grants the first N requests of a
world's life (creation, 45 bodies, 60 steps with the device arena regrowing past its
first capacities) and refuses the rest.  Every run must end normally: either the world
was not created, or it reports B2_STATUS_OUT_OF_HOST_MEMORY (-2) and stopped, and no
host memory is leaked once it is destroyed.  The failures are made on the host; no GPU
fault is involved."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory, gpu):
    import box2c_gb300
    lib = box2c_gb300.build()
    exe = str(tmp_path_factory.mktemp("alloc") / "alloc_fault")
    subprocess.run(["gcc", "-std=gnu17", "-O1", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c", "alloc_fault.c"), "-L", os.path.dirname(lib), "-lbox2d_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True, capture_output=True)

    def run(grant):
        r = subprocess.run([exe, str(grant)], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, f"grant {grant}: exit {r.returncode}\n{r.stdout}{r.stderr}"
        return dict(kv.split("=") for kv in r.stdout.split())

    return run


def test_allocator_hook_carries_the_library_memory(harness):
    out = harness(-1)
    assert out["world"] == "1" and out["bodies"] == "45" and out["status"] == "0"
    assert int(out["calls"]) > 0 and out["refused"] == "0"
    assert out["leaked"] == "0"


def test_refused_requests_fail_the_world_cleanly(harness):
    total = int(harness(-1)["calls"])
    grants = sorted(set(list(range(0, 24)) + [int(total * f) for f in (0.1, 0.25, 0.4, 0.5, 0.6, 0.75, 0.9, 0.97)]
                        + [total - 2, total - 1]))
    failed_in_step = 0
    for g in grants:
        out = harness(g)
        if out["refused"] == "0":
            continue
        assert out["world"] == "0" or out["status"] == "-2", (g, out)
        assert out["leaked"] == "0", (g, out)
        failed_in_step += out["world"] == "1" and out["bodies"] == "45"
    assert failed_in_step > 0  # some refusals came during the steps, not only at creation
