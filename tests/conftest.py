"""Shared fixtures: the GPU backend, the plain-C oracle and (in the build container
only) the reference build.  The oracle and reference are checkers, never the product."""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

from box2c_gb300.capi import Backend  # noqa: E402

ORACLE_DIR = os.path.join(REPO, "oracle")
REF_SRC = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _make(args):
    subprocess.run(["make", "-s", "-j8"] + args, cwd=REPO, check=True, capture_output=True)


@pytest.fixture(scope="session")
def oracle():
    _make(["-f", "oracle/Makefile"])
    b = os.path.join(ORACLE_DIR, "_build")
    return Backend(os.path.join(b, "liboracle.so"), os.path.join(b, "liboracle_scenes.so"), "oracle")


@pytest.fixture(scope="session")
def oracle64():
    _make(["-f", "oracle/Makefile"])
    b = os.path.join(ORACLE_DIR, "_build")
    return Backend(os.path.join(b, "liboracle64.so"), os.path.join(b, "liboracle64_scenes.so"), "oracle64")


@pytest.fixture(scope="session")
def oracle_atan():
    """The float oracle with the library's own atan2 in place of the C library's (joint
    springs and limits are then comparable bit for bit with the device)."""
    _make(["-f", "oracle/Makefile"])
    b = os.path.join(ORACLE_DIR, "_build")
    return Backend(os.path.join(b, "liboracle_atan.so"), os.path.join(b, "liboracle_atan_scenes.so"), "oracle_atan")


@pytest.fixture(scope="session")
def reference():
    if not os.path.isdir(os.path.join(REF_SRC, "src")):
        pytest.skip("reference sources not present on this machine")
    _make(["-f", "oracle/Makefile.ref", f"REF={REF_SRC}"])
    b = os.path.join(ORACLE_DIR, "_ref")
    return Backend(os.path.join(b, "libb2ref.so"), os.path.join(b, "libb2ref_scenes.so"), "reference")


@pytest.fixture(scope="session")
def gpu():
    import box2c_gb300
    box2c_gb300.build()
    return box2c_gb300.load()
