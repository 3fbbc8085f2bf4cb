"""Unit checks of the step adjoint's pieces (tests/cuda/*.cu): every row VJP, the
integration and finalisation VJPs, the row-preparation VJP and the dual-number
manifold Jacobian against central differences of the float routines they
differentiate.  Each check is a small CUDA program compiled here with nvcc."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")


@pytest.mark.parametrize("name", ["vjp_check", "jacobian_check"])
def test_adjoint_unit_check(name, tmp_path):
    exe = str(tmp_path / name)
    subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "--fmad=false", "-std=c++17",
                    "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "box2c_gb300", "csrc"),
                    os.path.join(HERE, "cuda", name + ".cu"), "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    bad = [line for line in r.stdout.splitlines() if "MISMATCH" in line or "mismatch" in line]
    assert not bad, "\n".join(bad)
    assert "status no error" in r.stdout
