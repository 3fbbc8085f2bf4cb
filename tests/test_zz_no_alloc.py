"""b2SolveContactsNoAlloc against b2SolveContacts on the same captured solver inputs.

Collected last so that it also runs after every other GPU test in the same process;
it passes alone in a fresh process as well.  Tolerance: none, results must be
bit-identical (both entry points run the same kernels on the same inputs).
"""
import ctypes as C

import numpy as np
import pytest

from box2c_gb300.capi import ContactSolveDesc, bind_solve_api
from tests.test_gpu_solve_api import DT, SUBSTEPS, capture_step, make_desc

MAX_CONTACTS = 16384  # B2_SOLVE_NOALLOC_MAX_CONTACTS, include/box2d/gpu.h
TOO_LARGE = -2  # B2_SOLVE_NOALLOC_TOO_LARGE


def _bind(lib):
    bind_solve_api(lib)
    lib.b2SolveContactsNoAlloc.argtypes = [C.POINTER(ContactSolveDesc)]
    lib.b2SolveContactsNoAlloc.restype = C.c_int


def _run(torch, fn, cap):
    d, t = make_desc(torch, cap, "cuda:0")
    rc = fn(C.byref(d))
    torch.cuda.synchronize()
    assert rc == 0
    return t["statesIn"].cpu().numpy(), t["manifoldsIn"].cpu().numpy()


def _capture(oracle, world, warm):
    oracle.step(world, DT, SUBSTEPS, warm)
    cap = capture_step(oracle, world)
    oracle.destroy(world)
    return cap


@pytest.mark.gpu
def test_no_alloc_matches_allocating_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    _bind(gpu.lib)
    big = _capture(oracle, oracle.pyramid(40, 0.01, 77), 25)
    small = _capture(oracle, oracle.pyramid(20), 40)
    assert 0 < len(small["contactBodies"]) < len(big["contactBodies"]) <= MAX_CONTACTS
    # two calls in a row (a larger then a smaller set, so the second reuses rows the
    # first left behind), each against b2SolveContacts on the same inputs
    for cap in (big, small):
        want = _run(torch, gpu.lib.b2SolveContacts, cap)
        got = _run(torch, gpu.lib.b2SolveContactsNoAlloc, cap)
        assert np.array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
        assert np.array_equal(got[1], want[1])


@pytest.mark.gpu
def test_no_alloc_rejects_oversized_set(gpu):
    torch = pytest.importorskip("torch")
    _bind(gpu.lib)
    n = MAX_CONTACTS + 1
    states = torch.zeros((1, 8), dtype=torch.float32, device="cuda:0")
    body4 = torch.zeros((1, 4), dtype=torch.float32, device="cuda:0")
    pairs = torch.full((n, 2), -1, dtype=torch.int32, device="cuda:0")
    mix = torch.zeros((n, 2), dtype=torch.float32, device="cuda:0")
    d = ContactSolveDesc()
    d.states = states.data_ptr()
    d.massData = d.forces = d.damping = body4.data_ptr()
    d.bodies = None
    d.bodyCount = 0
    d.contactBodies = pairs.data_ptr()
    d.contactMix = mix.data_ptr()
    d.manifolds = mix.data_ptr()  # never read: the call is rejected before any launch
    d.contactCount = n
    for c in range(1, 13):
        d.colorStart[c] = n
    d.timeStep = DT
    d.subStepCount = SUBSTEPS
    assert gpu.lib.b2SolveContactsNoAlloc(C.byref(d)) == TOO_LARGE
    torch.cuda.synchronize()


def _default_pool_used_high(reset):
    """High-water mark of the current device's default memory pool (the pool that
    stream-ordered allocations come from), read through the CUDA runtime the process
    has loaded; reset to the current use first when `reset`."""
    lib = None
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart.so" in line:
                lib = line.split()[-1]
                break
    if lib is None:
        pytest.skip("no shared CUDA runtime loaded in this process")
    rt = C.CDLL(lib)
    pool = C.c_void_p()
    dev = C.c_int()
    assert rt.cudaGetDevice(C.byref(dev)) == 0
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    used_high = 0x8  # cudaMemPoolAttrUsedMemHigh
    if reset:
        zero = C.c_uint64(0)
        assert rt.cudaMemPoolSetAttribute(pool, used_high, C.byref(zero)) == 0
    value = C.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, used_high, C.byref(value)) == 0
    return value.value


@pytest.mark.gpu
def test_no_alloc_takes_no_device_memory(gpu, oracle):
    """The property the entry point exists for: across a b2SolveContactsNoAlloc call the
    default pool's high-water mark stays at the use it was reset to, while
    b2SolveContacts on the same inputs raises it (its rows come from that pool)."""
    torch = pytest.importorskip("torch")
    _bind(gpu.lib)
    cap = _capture(oracle, oracle.pyramid(20), 40)
    _run(torch, gpu.lib.b2SolveContactsNoAlloc, cap)  # first call on the device: set-up
    d, t = make_desc(torch, cap, "cuda:0")
    torch.cuda.synchronize()
    base = _default_pool_used_high(reset=True)  # the pool's use now (live worlds' arenas)
    assert gpu.lib.b2SolveContactsNoAlloc(C.byref(d)) == 0
    torch.cuda.synchronize()
    assert _default_pool_used_high(reset=False) == base
    assert gpu.lib.b2SolveContacts(C.byref(d)) == 0
    torch.cuda.synchronize()
    assert _default_pool_used_high(reset=False) > base
