"""CPU: libhsr.so builds, loads and exports every entry point include/hsr.h declares; without
a CUDA device the calls fail with a status code (there is no CPU fallback)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hsr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hsr_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    import build_lib

    return build_lib.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("hsr_init", "hsr_draw", "hsr_draw_batch", "hsr_mesh_upload", "hsr_texture_upload",
                 "hsr_target_create", "hsr_target_clear", "hsr_target_download"):
        assert must in syms


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_no_device_means_error_not_fallback(libpath):
    import torch  # noqa: F401  (only to know whether this host has a device)

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import hsr

    L = hsr.lib()
    assert L.hsr_abi_version() == 2
    rc = L.hsr_init(0)
    assert rc == hsr.ERR_CUDA
    assert b"device" in L.hsr_last_error() or len(L.hsr_last_error()) > 0
    h = ctypes.c_uint64()
    assert L.hsr_target_create(16, 16, ctypes.byref(h)) == hsr.ERR_NOT_INITIALIZED


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the ABI structs have the C sizes and offsets."""
    import shutil
    import subprocess

    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    import hsr

    checks = {
        "hsr_draw_desc": (hsr.DrawDesc, ["uniforms", "prim_base", "clear_rgba"]),
        "hsr_request": (hsr.Request, ["uniforms", "clear_rgba", "shadow_clear_depth", "out_rgba", "out_prim"]),
        "hsr_request_status": (hsr.RequestStatus, ["deferred", "submit_ms", "done_ms"]),
        "hsr_server_config": (hsr.ServerConfig, ["max_batch", "slots"]),
        "hsr_timing": (hsr.Timing, ["launches", "h2d_bytes", "clipped_faces", "fragments", "raster_pixels", "tiles",
                                     "payload_bytes"]),
        "hsr_stats": (hsr.Stats, ["kernel_launches"]),
        "hsr_tuning": (hsr.Tuning, ["bin_factor"]),
        "hsr_transform": (hsr.Transform, ["rotation", "scale"]),
        "hsr_scene_params": (hsr.SceneParams, ["width", "model", "enable_shadow", "gloss", "bump_scale"]),
        "hsr_camera_motion": (hsr.CameraMotion, ["pan", "dolly"]),
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hsr.h"', "int main(void) {"]
    for cname, (_, fields) in checks.items():
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    exp = []
    for _, (cls, fields) in checks.items():
        exp.append(ctypes.sizeof(cls))
        exp.extend(getattr(cls, f).offset for f in fields)
    assert got == exp
    assert ctypes.sizeof(hsr.Request) - hsr.Request.uniforms.offset >= hsr.SHADER_DATA_DTYPE.itemsize
