"""The C-ABI library builds, loads without a GPU, and exports every function declared in
include/box2d/*.h (no compute call is made here)."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(REPO, "include", "box2d")


def declared_functions():
    names = set()
    for f in sorted(os.listdir(INC)):
        text = open(os.path.join(INC, f)).read()
        # B2_API declarations and the plain prototypes of inspect.h / gpu.h
        for m in re.finditer(r"B2_API\s+[\w\s\*]+?\b(b2\w+)\s*\(", text):
            names.add(m.group(1))
        if f in ("inspect.h", "gpu.h"):
            for m in re.finditer(r"^\s*(?:int|void|float|bool|b2\w+)\s*\*?\s*(b2\w+)\s*\(", text, re.M):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import box2c_gb300
    path = box2c_gb300.build()
    return C.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)


def test_headers_declare_the_step_path():
    names = declared_functions()
    for required in ("b2CreateWorld", "b2World_Step", "b2CreateBody", "b2CreatePolygonShape",
                     "b2CreateRevoluteJoint", "b2Body_GetPosition", "b2World_InspectContacts"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert missing == [], f"not exported: {missing}"


def test_no_device_means_no_world(lib):
    """Without a GPU the library refuses to create a world instead of falling back."""
    lib.b2gd_device_ok.restype = C.c_int
    if lib.b2gd_device_ok():
        pytest.skip("a GPU is visible")
    from box2c_gb300.capi import WorldId

    class WorldDef(C.Structure):
        _fields_ = [("gx", C.c_float), ("gy", C.c_float)] + [(f"f{i}", C.c_float) for i in range(7)] + \
                   [("s", C.c_bool), ("c", C.c_bool), ("wc", C.c_int32), ("e", C.c_void_p), ("fi", C.c_void_p),
                    ("u", C.c_void_p), ("iv", C.c_int32)]
    lib.b2DefaultWorldDef.restype = WorldDef
    lib.b2CreateWorld.restype = WorldId
    lib.b2CreateWorld.argtypes = [C.c_void_p]
    d = lib.b2DefaultWorldDef()
    w = lib.b2CreateWorld(C.byref(d))
    assert w.index1 == 0


def test_manifold_functions_match_reference_golden(lib):
    """The library's b2Collide* host functions run the manifold code the narrowphase kernel
    runs (box2c_gb300/csrc/b2g_collide.h, one source for host and device); on the seeded
    shape pairs they must give the reference's manifolds bit for bit."""
    import numpy as np
    from tests.golden.shapes import Manifold, manifold_array, random_pairs
    from box2c_gb300.capi import Transform
    golden = np.load(os.path.join(REPO, "tests", "golden", "manifolds.npz"))["outputs"]
    pairs = random_pairs(seed=7, count=len(golden))
    kinds = set()
    for k, (kind, a, xa, b, xb) in enumerate(pairs):
        fn = getattr(lib, kind)
        fn.restype = Manifold
        fn.argtypes = [C.c_void_p, Transform, C.c_void_p, Transform]
        got = manifold_array(fn(C.addressof(a), xa, C.addressof(b), xb))
        assert np.array_equal(got.view(np.uint32), golden[k].view(np.uint32)), (k, kind)
        kinds.add(kind)
    assert len(kinds) >= 4


def test_smooth_segment_manifolds_match_reference_golden(lib):
    """The library's chain-link manifold functions (the narrowphase kernel's code, compiled
    for the host) against the reference on seeded links and shapes: manifolds and the
    closest-feature cache, from an empty and from a warmed cache, bit for bit."""
    import numpy as np
    from tests.golden.shapes import collide_smooth, random_smooth_pairs
    golden = np.load(os.path.join(REPO, "tests", "golden", "smooth_manifolds.npz"))["outputs"]
    for k, entry in enumerate(random_smooth_pairs(seed=11, count=len(golden))):
        got = collide_smooth(lib, entry)
        assert np.array_equal(got.view(np.uint32), golden[k].view(np.uint32)), (k, entry[0], got, golden[k])
