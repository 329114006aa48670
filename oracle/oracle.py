"""ctypes binding of oracle/liboracle.so — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of bench.py use it,
always as the checker (or the timed CPU baseline), never as the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)


class _Mesh(ctypes.Structure):
    _fields_ = [("pos", _f32p), ("npos", ctypes.c_int32), ("nrm", _f32p), ("nnrm", ctypes.c_int32),
                ("uv", _f32p), ("nuv", ctypes.c_int32), ("faces", _i32p), ("nfaces", ctypes.c_int32)]


class _Tex(ctypes.Structure):
    _fields_ = [("data", _u8p), ("w", ctypes.c_int32), ("h", ctypes.c_int32), ("bpp", ctypes.c_int32)]


class _Target(ctypes.Structure):
    _fields_ = [("w", ctypes.c_int32), ("h", ctypes.c_int32), ("color", _u8p), ("depth", _f32p), ("prim", _u32p)]


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.hsro_draw.restype = ctypes.c_int
        L.hsro_draw.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_int32, ctypes.c_void_p,
                                ctypes.POINTER(_Tex), ctypes.POINTER(_Tex), ctypes.POINTER(_Target),
                                ctypes.POINTER(_Target), ctypes.c_uint32]
        L.hsro_clear.restype = None
        L.hsro_clear.argtypes = [ctypes.POINTER(_Target), _u8p, ctypes.c_float]
        L.hsro_bench_frames.restype = ctypes.c_double
        L.hsro_bench_frames.argtypes = [ctypes.POINTER(_Mesh), ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.POINTER(_Tex), ctypes.POINTER(_Tex),
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32]
        L.hsro_no_contraction.restype = ctypes.c_int
        if not L.hsro_no_contraction():
            raise RuntimeError("liboracle.so was built with floating-point contraction")
        _lib = L
    return _lib


class Buffers:
    """Host render target: RGBA8 colour, FP32 depth, u32 prim ids, row 0 = bottom."""

    def __init__(self, w: int, h: int, rgba=(0, 0, 0, 1), depth=np.finfo(np.float32).max):
        self.w, self.h = w, h
        self.color = np.empty((h, w, 4), np.uint8)
        self.depth = np.empty((h, w), np.float32)
        self.prim = np.empty((h, w), np.uint32)
        self.clear(rgba, depth)

    def clear(self, rgba, depth) -> None:
        self.color[:] = np.array(rgba, np.uint8)
        self.depth[:] = np.float32(depth)
        self.prim[:] = 0

    def _c(self) -> _Target:
        return _Target(self.w, self.h, self.color.ctypes.data_as(_u8p), self.depth.ctypes.data_as(_f32p),
                       self.prim.ctypes.data_as(_u32p))


def _tex(t):
    if t is None:
        return None
    d = np.ascontiguousarray(t.data)
    return _Tex(d.ctypes.data_as(_u8p), t.w, t.h, t.bpp), d


def _mesh(mesh):
    keep = [np.ascontiguousarray(mesh.pos, np.float32), np.array(mesh.nrm, np.float32, copy=True),
            np.ascontiguousarray(mesh.uv, np.float32), np.ascontiguousarray(mesh.faces, np.int32)]
    m = _Mesh(keep[0].ctypes.data_as(_f32p), len(keep[0]), keep[1].ctypes.data_as(_f32p), len(keep[1]),
              keep[2].ctypes.data_as(_f32p), len(keep[2]), keep[3].ctypes.data_as(_i32p), len(keep[3]))
    return m, keep


def draw(mesh, shader: int, sd: np.ndarray, target: Buffers, diffuse=None, normal=None,
         shadow_map: Buffers | None = None, prim_base: int = 0) -> None:
    """One graphics_draw_triangle(); the mesh's normals are copied (the oracle normalises its
    copy in place, as Model::normal does)."""
    L = lib()
    m, keep = _mesh(mesh)
    sdb = np.ascontiguousarray(sd)
    td = _tex(diffuse)
    tn = _tex(normal)
    sm = shadow_map._c() if shadow_map is not None else None
    tg = target._c()
    rc = L.hsro_draw(ctypes.byref(m), shader, sdb.ctypes.data_as(ctypes.c_void_p),
                     ctypes.byref(td[0]) if td else None, ctypes.byref(tn[0]) if tn else None,
                     ctypes.byref(sm) if sm is not None else None, ctypes.byref(tg), prim_base)
    if rc != 0:
        raise ValueError(f"hsro_draw failed ({rc})")
    del keep


def render_frame(frame) -> dict:
    """DrawModel::draw order: shadow pass into a shadow target, then the main pass."""
    from hsr import scenes

    out = {}
    sm = None
    if frame.shadow_size[0] > 0:
        sm = Buffers(frame.shadow_size[0], frame.shadow_size[1], frame.shadow_clear_rgba, frame.shadow_clear_depth)
        draw(frame.mesh, scenes.SHADOW, frame.sd, sm, frame.diffuse, frame.normal)
        out["shadow"] = sm
    main = Buffers(frame.width, frame.height, frame.clear_rgba, frame.clear_depth)
    draw(frame.mesh, frame.shader, frame.sd, main, frame.diffuse, frame.normal, shadow_map=sm)
    out["main"] = main
    return out


def bench_frames(frame, frames_each: int, threads: int) -> float:
    """Wall seconds for `threads` threads each rendering `frames_each` frames."""
    L = lib()
    m, keep = _mesh(frame.mesh)
    sdb = np.ascontiguousarray(frame.sd)
    td = _tex(frame.diffuse)
    tn = _tex(frame.normal)
    s = L.hsro_bench_frames(ctypes.byref(m), frame.shader, sdb.ctypes.data_as(ctypes.c_void_p),
                            ctypes.byref(td[0]) if td else None, ctypes.byref(tn[0]) if tn else None,
                            frame.width, frame.height, frame.shadow_size[0], frame.shadow_size[1],
                            frames_each, threads)
    del keep
    if s < 0:
        raise RuntimeError("hsro_bench_frames failed")
    return s
