"""CPU: the drop-in shim (graphics_draw_triangle over the C ABI) compiles against the
reference's own headers and links with the reference's sources in place of graphics.cpp.
Runs only where the reference sources are present."""
import os
import subprocess

import pytest

import refjob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not refjob.have_reference(), reason="reference sources not present on this host")
def test_shim_links_into_the_reference_build():
    import build_lib

    build_lib.build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "shim", f"REF={refjob.REF_DIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_harness_gpu")
    assert os.path.exists(exe)
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    assert "graphics_draw_triangle(DrawData*)" in syms
