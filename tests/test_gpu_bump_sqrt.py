"""GPU: NormalMapShader's bump height, (float)sqrt(1.0 - saturate(.)) evaluated in double by the
reference (IShader.cpp:143), is computed in single precision on the device (bump_height in
hsr_device.cuh).  This compiles a small checker against that device function and runs it over
every float in [0, 1]: the results must equal the double expression bit for bit."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bump_height_equals_double_expression_for_every_float(tmp_path):
    import build_lib

    nvcc = build_lib.nvcc()
    exe = tmp_path / "bump_z_check"
    subprocess.run([nvcc, build_lib.ARCH, "-O3", "-std=c++17", "--fmad=false", "--prec-div=true", "--prec-sqrt=true",
                    "--ftz=false", "-I", os.path.join(ROOT, "hana-softwarerenderer_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cuda", "bump_z_check.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    status, count = r.stdout.split()[:2]
    assert status == "cudaSuccess", r.stdout
    assert int(count) == 0, r.stdout
