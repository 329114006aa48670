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
    assert L.hsr_abi_version() == 1
    rc = L.hsr_init(0)
    assert rc == hsr.ERR_CUDA
    assert b"device" in L.hsr_last_error() or len(L.hsr_last_error()) > 0
    h = ctypes.c_uint64()
    assert L.hsr_target_create(16, 16, ctypes.byref(h)) == hsr.ERR_NOT_INITIALIZED
