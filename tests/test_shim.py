"""CPU: the drop-in shim (graphics_draw_triangle over the C ABI) compiles against the
reference's own headers and links with the reference's sources in place of graphics.cpp,
and — linked over a host stand-in of the C ABI (oracle/hsr_host_abi.c) — draws the
reference's jobs exactly as graphics.cpp does.  Runs only where the reference sources are
present."""
import os
import subprocess

import numpy as np
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


def _golden_module():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def shim_host():
    """The reference harness twice: with its own graphics.cpp (ref_harness) and with the shim in
    its place over a host stand-in of the C ABI that draws with the oracle (ref_harness_shim_host)."""
    if not refjob.have_reference():
        pytest.skip("reference sources not present on this host")
    import build_lib

    build_lib.build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "shim-host", f"REF={refjob.REF_DIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return refjob.SHIM_HOST_HARNESS


def _same(ref, got, label):
    assert ref.keys() == got.keys(), label
    for k in ref:
        for p in ("depth", "color"):
            assert np.array_equal(ref[k][p].view(np.uint8), got[k][p].view(np.uint8)), (label, k, p)


def test_shim_draws_like_graphics_cpp(shim_host):
    """Every shader of the reference, the shadow pass, clipping, ties, 1- and 3-byte maps and
    the clear states, drawn by the reference's application code through the shim: depth and
    RGBA8 bit for bit equal to the same jobs drawn by graphics.cpp.  (The stand-in draws with
    the oracle, so this checks the shim's translation, not the GPU kernels.)"""
    from hsr import scenes

    g = _golden_module()
    frames = [f for f in g.fixtures() if f.shader != scenes.FLAT]
    assert {f.shader for f in frames} == set(range(7))
    for fr in frames:
        _same(refjob.run(fr), refjob.run(fr, harness=shim_host), fr.name)


@pytest.mark.skipif(not refjob.have_assets(), reason="bundled assets not present (make -C oracle assets)")
def test_shim_draws_bundled_models_like_graphics_cpp(shim_host):
    """african_head and diablo3_pose from their files: the normals the shim reads through
    Model::normal on each draw (the shadow pass, then the main pass) drift as the reference's
    own reads make them drift, so the drawn frames are bit for bit those of graphics.cpp."""
    g = _golden_module()
    for model, shader, shadow in g.ASSET_SCENES:
        fr = g.asset_frame(model, shader, shadow)
        obj = refjob.asset(model, ".obj")
        _same(refjob.run(fr, obj_path=obj), refjob.run(fr, obj_path=obj, harness=shim_host), fr.name)


def test_shim_refuses_a_shader_it_does_not_implement(shim_host):
    """An IShader subclass the library has no kernel for (the harness's PrimIdShader) is
    reported and not drawn: the target keeps its clear values (there is no CPU fallback)."""
    from hsr import scenes

    fr = scenes.sphere_frame(3, 64, 48, shader=scenes.FLAT, seed=5)
    got = refjob.run(fr, harness=shim_host)["main"]
    assert np.all(got["depth"] == np.float32(fr.clear_depth))
    assert np.all(got["color"] == np.array(fr.clear_rgba, np.uint8))
