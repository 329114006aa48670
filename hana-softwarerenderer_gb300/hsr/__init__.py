"""ctypes binding of libhsr.so, the GB300 draw path behind the C ABI in include/hsr.h.

The library is the product; this module only marshals numpy arrays into its entry points.
It never renders on the CPU: if libhsr.so is missing or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .uniforms import SHADER_DATA_DTYPE  # noqa: F401  (re-exported)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libhsr.so")

# status codes (include/hsr.h)
OK, ERR_INVALID_ARG, ERR_UNKNOWN_SHADER, ERR_BIN_OVERFLOW, ERR_OUT_OF_MEMORY, ERR_TIMEOUT, ERR_CUDA, \
    ERR_NOT_INITIALIZED, ERR_BAD_HANDLE, ERR_BUSY = range(10)
DRAW_CLEAR = 1

_u8p = ctypes.POINTER(ctypes.c_uint8)
_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class HsrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hsr error {code}: {msg}")
        self.code = code


class DrawDesc(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint64), ("shader", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("diffuse", ctypes.c_uint64), ("normal", ctypes.c_uint64), ("target", ctypes.c_uint64),
                ("shadow_map", ctypes.c_uint64), ("uniforms", ctypes.c_void_p), ("prim_base", ctypes.c_uint32),
                ("clear_depth", ctypes.c_float), ("clear_rgba", ctypes.c_uint8 * 4)]


class Tuning(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("warps_per_cta", ctypes.c_int32),
                ("bin_factor", ctypes.c_float)]


# kernels of one launch sequence, in launch order (hsr_timing.kernel_ms)
KERNELS = ("vertex", "cull", "emit", "clip", "split", "scan", "scatter", "raster")


class Timing(ctypes.Structure):
    _fields_ = [("batch_ms", ctypes.c_float), ("kernel_ms", ctypes.c_float * len(KERNELS)),
                ("launches", ctypes.c_uint32), ("views", ctypes.c_uint32), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64), ("pixels", ctypes.c_uint64), ("shaded_pixels", ctypes.c_uint64),
                ("records", ctypes.c_uint64), ("bin_pairs", ctypes.c_uint64), ("faces", ctypes.c_uint64),
                ("vertices", ctypes.c_uint64), ("normals", ctypes.c_uint64), ("clipped_faces", ctypes.c_uint64),
                ("fragments", ctypes.c_uint64), ("raster_pixels", ctypes.c_uint64), ("tiles", ctypes.c_uint64),
                ("split_triangles", ctypes.c_uint64), ("payload_bytes", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("records", ctypes.c_uint64), ("clipped_faces", ctypes.c_uint64), ("bin_pairs", ctypes.c_uint64),
                ("tiles", ctypes.c_uint64), ("retries", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_int32), ("slots", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint64), ("shader", ctypes.c_int32), ("diffuse", ctypes.c_uint64),
                ("normal", ctypes.c_uint64), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("shadow_size", ctypes.c_int32), ("uniforms", ctypes.c_float * 121),
                ("clear_rgba", ctypes.c_uint8 * 4), ("clear_depth", ctypes.c_float),
                ("shadow_clear_rgba", ctypes.c_uint8 * 4), ("shadow_clear_depth", ctypes.c_float),
                ("out_rgba", ctypes.c_void_p), ("out_depth", ctypes.c_void_p), ("out_prim", ctypes.c_void_p)]


class Transform(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("rotation", ctypes.c_float * 3), ("scale", ctypes.c_float * 3)]


class CameraMotion(ctypes.Structure):
    _fields_ = [("orbit", ctypes.c_float * 2), ("pan", ctypes.c_float * 2), ("dolly", ctypes.c_float)]


class SceneParams(ctypes.Structure):
    _fields_ = [("camera_position", ctypes.c_float * 3), ("camera_target", ctypes.c_float * 3),
                ("light_position", ctypes.c_float * 3), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("model", Transform), ("enable_shadow", ctypes.c_int32), ("material_color", ctypes.c_float * 4),
                ("material_specular", ctypes.c_float * 4), ("gloss", ctypes.c_float), ("bump_scale", ctypes.c_float)]


class RequestStatus(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("batch", ctypes.c_uint32), ("batch_requests", ctypes.c_uint32),
                ("deferred", ctypes.c_uint32), ("submit_ms", ctypes.c_double), ("launch_ms", ctypes.c_double),
                ("done_ms", ctypes.c_double)]


_lib = None


def lib_path() -> str:
    return LIB_PATH


def lib():
    """Load libhsr.so (built in-tree by build_lib.py); raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "hsr_init": ([ctypes.c_int], ctypes.c_int),
        "hsr_shutdown": ([], ctypes.c_int),
        "hsr_last_error": ([], ctypes.c_char_p),
        "hsr_abi_version": ([], ctypes.c_int),
        "hsr_mesh_upload": ([_f32p, ctypes.c_int32, _f32p, ctypes.c_int32, _f32p, ctypes.c_int32, _i32p,
                             ctypes.c_int32, _u64p], ctypes.c_int),
        "hsr_mesh_update_normals": ([ctypes.c_uint64, _f32p, ctypes.c_int32], ctypes.c_int),
        "hsr_mesh_release": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_texture_upload": ([_u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _u64p], ctypes.c_int),
        "hsr_texture_release": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_target_create": ([ctypes.c_int32, ctypes.c_int32, _u64p], ctypes.c_int),
        "hsr_target_release": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_target_clear": ([ctypes.c_uint64, _u8p, ctypes.c_float], ctypes.c_int),
        "hsr_target_upload": ([ctypes.c_uint64, _u8p, _f32p, _u32p], ctypes.c_int),
        "hsr_target_download": ([ctypes.c_uint64, _u8p, _f32p, _u32p], ctypes.c_int),
        "hsr_draw": ([ctypes.POINTER(DrawDesc)], ctypes.c_int),
        "hsr_draw_batch": ([ctypes.POINTER(DrawDesc), ctypes.c_int32], ctypes.c_int),
        "hsr_draw_noalloc": ([ctypes.POINTER(DrawDesc)], ctypes.c_int),
        "hsr_synchronize": ([], ctypes.c_int),
        "hsr_get_tuning": ([ctypes.POINTER(Tuning)], ctypes.c_int),
        "hsr_set_tuning": ([ctypes.POINTER(Tuning)], ctypes.c_int),
        "hsr_get_stats": ([ctypes.POINTER(Stats)], ctypes.c_int),
        "hsr_set_profiling": ([ctypes.c_int], ctypes.c_int),
        "hsr_autotune": ([ctypes.POINTER(DrawDesc), ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Tuning)],
                         ctypes.c_int),
        "hsr_last_timing": ([ctypes.POINTER(Timing)], ctypes.c_int),
        "hsr_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
        "hsr_host_free": ([ctypes.c_void_p], ctypes.c_int),
        "hsr_plan_create": ([ctypes.POINTER(DrawDesc), ctypes.c_int32, _u64p], ctypes.c_int),
        "hsr_plan_set_uniforms": ([ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p], ctypes.c_int),
        "hsr_plan_launch": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_plan_wait": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_plan_release": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_server_create": ([ctypes.POINTER(ServerConfig), _u64p], ctypes.c_int),
        "hsr_server_submit": ([ctypes.c_uint64, ctypes.POINTER(Request), _u64p], ctypes.c_int),
        "hsr_server_poll": ([ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(RequestStatus)], ctypes.c_int),
        "hsr_server_wait": ([ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(RequestStatus)],
                            ctypes.c_int),
        "hsr_server_now_ms": ([ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "hsr_server_destroy": ([ctypes.c_uint64], ctypes.c_int),
        "hsr_server_inject_alloc_failures": ([ctypes.c_uint64, ctypes.c_int32], ctypes.c_int),
        "hsr_set_fault_injection": ([ctypes.c_uint32, ctypes.c_int32], ctypes.c_int),
        "hsr_shader_data_build": ([ctypes.POINTER(SceneParams), ctypes.c_void_p], ctypes.c_int),
        "hsr_model_matrix": ([ctypes.POINTER(Transform), _f32p], ctypes.c_int),
        "hsr_matrix_invert": ([_f32p, _f32p], ctypes.c_int),
        "hsr_camera_update": ([_f32p, _f32p, ctypes.POINTER(CameraMotion), _f32p, _f32p], ctypes.c_int),
        "hsr_obj_read": ([ctypes.c_char_p, ctypes.c_uint32, _f32p, _i32p, _f32p, _i32p, _f32p, _i32p, _i32p, _i32p],
                         ctypes.c_int),
        "hsr_tga_read": ([ctypes.c_char_p, ctypes.c_uint32, _u8p, _i32p, _i32p, _i32p], ctypes.c_int),
        "hsr_tga_write": ([ctypes.c_char_p, _u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
                          ctypes.c_int),
        "hsr_mesh_load_obj": ([ctypes.c_char_p, ctypes.c_uint32, _u64p], ctypes.c_int),
        "hsr_texture_load_tga": ([ctypes.c_char_p, ctypes.c_uint32, _u64p], ctypes.c_int),
        "hsr_target_present": ([ctypes.c_uint64, _u8p, ctypes.c_int32], ctypes.c_int),
        "hsr_target_write_tga": ([ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int32], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        raise HsrError(rc, lib().hsr_last_error().decode(errors="replace"))


def init(device: int = 0) -> None:
    check(lib().hsr_init(device))


def shutdown() -> None:
    check(lib().hsr_shutdown())


def synchronize() -> None:
    check(lib().hsr_synchronize())


def get_tuning() -> Tuning:
    t = Tuning()
    check(lib().hsr_get_tuning(ctypes.byref(t)))
    return t


def set_tuning(tile=None, ctas_per_sm=None, warps_per_cta=None, bin_factor=None) -> None:
    t = get_tuning()
    if tile is not None:
        t.tile = tile
    if ctas_per_sm is not None:
        t.ctas_per_sm = ctas_per_sm
    if warps_per_cta is not None:
        t.warps_per_cta = warps_per_cta
    if bin_factor is not None:
        t.bin_factor = bin_factor
    check(lib().hsr_set_tuning(ctypes.byref(t)))


def autotune(descs, reps: int = 3) -> dict:
    """Time the batch under each tuning candidate and keep the fastest (hsr_autotune)."""
    arr = (DrawDesc * len(descs))(*descs)
    t = Tuning()
    check(lib().hsr_autotune(arr, len(descs), reps, ctypes.byref(t)))
    return {k: getattr(t, k) for k, _ in Tuning._fields_}


def stats() -> dict:
    s = Stats()
    check(lib().hsr_get_stats(ctypes.byref(s)))
    return {k: int(getattr(s, k)) for k, _ in Stats._fields_}


FAULT_DEPENDENCY_STALL = 1
FAULT_SCAN_STALL = 2


def set_fault_injection(faults: int = 0, poll_limit: int = 0) -> None:
    """hsr_set_fault_injection: make a bounded device wait of hsr_draw / hsr_draw_batch run out
    (FAULT_* mask) after `poll_limit` polls (0: the default limit)."""
    check(lib().hsr_set_fault_injection(faults, poll_limit))


def set_profiling(on: bool) -> None:
    check(lib().hsr_set_profiling(1 if on else 0))


def last_timing() -> dict:
    t = Timing()
    check(lib().hsr_last_timing(ctypes.byref(t)))
    d = {k: (list(getattr(t, k)) if k == "kernel_ms" else getattr(t, k)) for k, _ in Timing._fields_}
    d["kernel_ms"] = dict(zip(KERNELS, d["kernel_ms"]))
    return d


class PinnedArray:
    """numpy view of page-locked host memory from hsr_host_alloc (freed on release())."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        check(lib().hsr_host_alloc(n, ctypes.byref(p)))
        self.ptr = p.value
        buf = (ctypes.c_uint8 * n).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def release(self) -> None:
        if self.ptr:
            self.array = None
            check(lib().hsr_host_free(ctypes.c_void_p(self.ptr)))
            self.ptr = None


# ---- uniforms (hsr_shader_data_build; host only, no device) ------------------------------
def transform(position=(0, 0, 0), rotation=(0, 0, 0), scale=(1, 1, 1)) -> Transform:
    t = Transform()
    t.position[:] = [float(v) for v in position]
    t.rotation[:] = [float(v) for v in rotation]
    t.scale[:] = [float(v) for v in scale]
    return t


def shader_data_build(camera_position, width: int, height: int, *, camera_target=(0, 0, 0), light=(2, 2, 2),
                      model: Transform | None = None, enable_shadow: bool = False, material_color=(1, 1, 1, 255),
                      material_specular=(1, 1, 1, 255), gloss: float = 50.0, bump_scale: float = 1.0) -> np.ndarray:
    """ShaderData as DrawModel::draw fills it (scene.h:55-71), built natively (hsr_uniforms.cpp)."""
    p = SceneParams()
    p.camera_position[:] = [float(v) for v in camera_position]
    p.camera_target[:] = [float(v) for v in camera_target]
    p.light_position[:] = [float(v) for v in light]
    p.width, p.height = width, height
    p.model = model if model is not None else transform()
    p.enable_shadow = 1 if enable_shadow else 0
    p.material_color[:] = [float(v) for v in material_color]
    p.material_specular[:] = [float(v) for v in material_specular]
    p.gloss, p.bump_scale = gloss, bump_scale
    sd = np.zeros((), SHADER_DATA_DTYPE)
    check(lib().hsr_shader_data_build(ctypes.byref(p), sd.ctypes.data))
    return sd


def model_matrix(t: Transform) -> np.ndarray:
    out = np.empty(16, np.float32)
    check(lib().hsr_model_matrix(ctypes.byref(t), out.ctypes.data_as(_f32p)))
    return out


def matrix_invert(m) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    out = np.empty(16, np.float32)
    check(lib().hsr_matrix_invert(a.ctypes.data_as(_f32p), out.ctypes.data_as(_f32p)))
    return out


def camera_update(position, target, orbit=(0.0, 0.0), pan=(0.0, 0.0), dolly: float = 0.0):
    """One step of the reference's orbital camera (Camera::update_transform, camera.cpp:63-70):
    returns the new (position, target) as float32 arrays."""
    p = np.ascontiguousarray(np.asarray(position, np.float32).reshape(3))
    t = np.ascontiguousarray(np.asarray(target, np.float32).reshape(3))
    m = CameraMotion((ctypes.c_float * 2)(*orbit), (ctypes.c_float * 2)(*pan), float(dolly))
    op, ot = np.empty(3, np.float32), np.empty(3, np.float32)
    check(lib().hsr_camera_update(p.ctypes.data_as(_f32p), t.ctypes.data_as(_f32p), ctypes.byref(m),
                                  op.ctypes.data_as(_f32p), ot.ctypes.data_as(_f32p)))
    return op, ot


# ---- asset files (hsr_obj_read / hsr_tga_read / hsr_tga_write; host only, no device) ----
OBJ_CORNER_NORMALS = 1
TGA_MODEL_FLIP = 1


def obj_earlier_draws(n: int) -> int:
    """Flag bits: with OBJ_CORNER_NORMALS, the normals of the draw after n earlier ones."""
    return (n & 255) << 8


def obj_read(path: str, flags: int = 0):
    """Parse an OBJ file like Model::Model: returns (pos (n,3) f32, nrm (n,3) f32, uv (n,2) f32,
    faces (nfaces,3,3) i32 with 0-based v/vt/vn per corner)."""
    L = lib()
    cnt = [ctypes.c_int32() for _ in range(4)]
    b = str(path).encode()
    check(L.hsr_obj_read(b, flags, None, ctypes.byref(cnt[0]), None, ctypes.byref(cnt[1]), None,
                         ctypes.byref(cnt[2]), None, ctypes.byref(cnt[3])))
    pos = np.empty((cnt[0].value, 3), np.float32)
    nrm = np.empty((cnt[1].value, 3), np.float32)
    uv = np.empty((cnt[2].value, 2), np.float32)
    faces = np.empty((cnt[3].value, 3, 3), np.int32)
    check(L.hsr_obj_read(b, flags, pos.ctypes.data_as(_f32p), ctypes.byref(cnt[0]), nrm.ctypes.data_as(_f32p),
                         ctypes.byref(cnt[1]), uv.ctypes.data_as(_f32p), ctypes.byref(cnt[2]),
                         faces.ctypes.data_as(_i32p), ctypes.byref(cnt[3])))
    return pos, nrm, uv, faces


def tga_read(path: str, flags: int = 0) -> np.ndarray:
    """Read a TGA file like TGAImage::read_tga_file: returns (h, w, bytespp) u8, the buffer
    layout (texel (x, y) at data[y, x], bytes B, G, R(, A))."""
    L = lib()
    w, h, bpp = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    b = str(path).encode()
    check(L.hsr_tga_read(b, flags, None, ctypes.byref(w), ctypes.byref(h), ctypes.byref(bpp)))
    out = np.empty((h.value, w.value, bpp.value), np.uint8)
    check(L.hsr_tga_read(b, flags, out.ctypes.data_as(_u8p), ctypes.byref(w), ctypes.byref(h), ctypes.byref(bpp)))
    return out


def tga_write(path: str, data: np.ndarray, rle: bool = False) -> None:
    """TGAImage::write_tga_file of an (h, w, bytespp) u8 buffer (top-left origin)."""
    d = np.ascontiguousarray(data, np.uint8)
    check(lib().hsr_tga_write(str(path).encode(), d.ctypes.data_as(_u8p), d.shape[1], d.shape[0], d.shape[2],
                              1 if rle else 0))


class Mesh:
    """A Model resident on the device (hsr_mesh_upload, or hsr_mesh_load_obj via from_obj)."""

    @classmethod
    def from_obj(cls, path: str, flags: int = 0) -> "Mesh":
        self = cls.__new__(cls)
        h = ctypes.c_uint64()
        check(lib().hsr_mesh_load_obj(str(path).encode(), flags, ctypes.byref(h)))
        self.handle = h.value
        self.nfaces = -1
        return self

    def __init__(self, mesh):
        pos = np.ascontiguousarray(mesh.pos, np.float32)
        nrm = np.ascontiguousarray(mesh.nrm, np.float32)
        uv = np.ascontiguousarray(mesh.uv, np.float32)
        faces = np.ascontiguousarray(mesh.faces, np.int32)
        h = ctypes.c_uint64()
        check(lib().hsr_mesh_upload(pos.ctypes.data_as(_f32p), len(pos), nrm.ctypes.data_as(_f32p), len(nrm),
                                    uv.ctypes.data_as(_f32p), len(uv), faces.ctypes.data_as(_i32p), len(faces),
                                    ctypes.byref(h)))
        self.handle = h.value
        self.nfaces = len(faces)

    def update_normals(self, nrm: np.ndarray) -> None:
        nrm = np.ascontiguousarray(nrm, np.float32)
        check(lib().hsr_mesh_update_normals(self.handle, nrm.ctypes.data_as(_f32p), len(nrm)))

    def release(self) -> None:
        if self.handle:
            check(lib().hsr_mesh_release(self.handle))
            self.handle = 0


class Texture:
    """A TGAImage resident on the device (hsr_texture_upload, or hsr_texture_load_tga via
    from_tga)."""

    @classmethod
    def from_tga(cls, path: str, flags: int = 0) -> "Texture":
        self = cls.__new__(cls)
        h = ctypes.c_uint64()
        check(lib().hsr_texture_load_tga(str(path).encode(), flags, ctypes.byref(h)))
        self.handle = h.value
        return self

    def __init__(self, tex):
        d = np.ascontiguousarray(tex.data, np.uint8)
        h = ctypes.c_uint64()
        check(lib().hsr_texture_upload(d.ctypes.data_as(_u8p), tex.w, tex.h, tex.bpp, ctypes.byref(h)))
        self.handle = h.value

    def release(self) -> None:
        if self.handle:
            check(lib().hsr_texture_release(self.handle))
            self.handle = 0


class Target:
    """A RenderBuffer (+ prim-id plane) resident on the device."""

    def __init__(self, w: int, h: int):
        hd = ctypes.c_uint64()
        check(lib().hsr_target_create(w, h, ctypes.byref(hd)))
        self.handle = hd.value
        self.w, self.h = w, h

    def clear(self, rgba=(0, 0, 0, 1), depth=float(np.finfo(np.float32).max)) -> None:
        c = (ctypes.c_uint8 * 4)(*rgba)
        check(lib().hsr_target_clear(self.handle, ctypes.cast(c, _u8p), depth))

    def upload(self, color=None, depth=None, prim=None) -> None:
        c = None if color is None else np.ascontiguousarray(color, np.uint8)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        p = None if prim is None else np.ascontiguousarray(prim, np.uint32)
        check(lib().hsr_target_upload(self.handle, c.ctypes.data_as(_u8p) if c is not None else None,
                                      d.ctypes.data_as(_f32p) if d is not None else None,
                                      p.ctypes.data_as(_u32p) if p is not None else None))

    def download(self, color=True, depth=True, prim=True, out=None):
        """Returns dict(color (h,w,4) u8, depth (h,w) f32, prim (h,w) u32); `out` may hold
        preallocated (pinned or not) arrays to fill."""
        out = out or {}
        c = out.get("color") if color else None
        d = out.get("depth") if depth else None
        p = out.get("prim") if prim else None
        if color and c is None:
            c = np.empty((self.h, self.w, 4), np.uint8)
        if depth and d is None:
            d = np.empty((self.h, self.w), np.float32)
        if prim and p is None:
            p = np.empty((self.h, self.w), np.uint32)
        check(lib().hsr_target_download(self.handle, c.ctypes.data_as(_u8p) if c is not None else None,
                                        d.ctypes.data_as(_f32p) if d is not None else None,
                                        p.ctypes.data_as(_u32p) if p is not None else None))
        return {"color": c, "depth": d, "prim": p}

    def present(self, channels: int = 3) -> np.ndarray:
        """The image window_draw_buffer shows: top-down rows, B, G, R (, 0) per pixel."""
        out = np.empty((self.h, self.w, channels), np.uint8)
        check(lib().hsr_target_present(self.handle, out.ctypes.data_as(_u8p), channels))
        return out

    def write_tga(self, path: str, rle: bool = False) -> None:
        check(lib().hsr_target_write_tga(self.handle, str(path).encode(), 1 if rle else 0))

    def release(self) -> None:
        if self.handle:
            check(lib().hsr_target_release(self.handle))
            self.handle = 0


def make_desc(mesh: Mesh, shader: int, sd: np.ndarray, target: Target, diffuse: Texture | None = None,
              normal: Texture | None = None, shadow_map: Target | None = None, prim_base: int = 0,
              clear=None, keep: list | None = None) -> DrawDesc:
    """Fill an hsr_draw_desc.  `clear=(rgba, depth)` fuses the clear into the draw.  The
    uniform record must stay alive until the draw call returns: it is appended to `keep`."""
    sdb = np.ascontiguousarray(np.asarray(sd, dtype=SHADER_DATA_DTYPE).reshape(()))
    if keep is not None:
        keep.append(sdb)
    d = DrawDesc()
    d.mesh = mesh.handle
    d.shader = shader
    d.flags = DRAW_CLEAR if clear is not None else 0
    d.diffuse = diffuse.handle if diffuse else 0
    d.normal = normal.handle if normal else 0
    d.target = target.handle
    d.shadow_map = shadow_map.handle if shadow_map else 0
    d.uniforms = sdb.ctypes.data
    d.prim_base = prim_base
    if clear is not None:
        rgba, depth = clear
        d.clear_depth = float(depth)
        for i in range(4):
            d.clear_rgba[i] = rgba[i]
    d._keep = sdb  # noqa: SLF001  keep the uniforms alive with the struct
    return d


def draw(desc: DrawDesc) -> None:
    check(lib().hsr_draw(ctypes.byref(desc)))


def draw_noalloc(desc: DrawDesc) -> None:
    """hsr_draw_noalloc: the draw on the library's fixed 128 MiB scratch, no allocation."""
    check(lib().hsr_draw_noalloc(ctypes.byref(desc)))


def draw_batch(descs) -> None:
    arr = (DrawDesc * len(descs))(*descs)
    check(lib().hsr_draw_batch(arr, len(descs)))


class Plan:
    """A batch recorded once into a CUDA graph (hsr_plan_create) and replayed; only the
    uniforms of its draws change between replays."""

    def __init__(self, descs):
        arr = (DrawDesc * len(descs))(*descs)
        h = ctypes.c_uint64()
        check(lib().hsr_plan_create(arr, len(descs), ctypes.byref(h)))
        self.handle = h.value
        self.n = len(descs)

    def set_uniforms(self, draw: int, sd) -> None:
        sdb = np.ascontiguousarray(np.asarray(sd, dtype=SHADER_DATA_DTYPE).reshape(()))
        check(lib().hsr_plan_set_uniforms(self.handle, draw, sdb.ctypes.data))

    def launch(self) -> None:
        check(lib().hsr_plan_launch(self.handle))

    def wait(self) -> None:
        check(lib().hsr_plan_wait(self.handle))

    def release(self) -> None:
        if self.handle:
            check(lib().hsr_plan_release(self.handle))
            self.handle = 0


_FLT_MAX = float(np.finfo(np.float32).max)


class Server:
    """Continuous-batching render server (hsr_server_*): requests are queued, admitted while
    the framebuffer pool has room, batched into launch sequences (`slots` batches in flight),
    and their colour / depth / prim ids copied into the arrays given at submission."""

    def __init__(self, pool_bytes: int, max_batch: int = 64, slots: int = 2):
        cfg = ServerConfig(pool_bytes, max_batch, slots)
        h = ctypes.c_uint64()
        check(lib().hsr_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h.value
        self._live: dict[int, tuple] = {}

    def submit(self, mesh: Mesh, shader: int, sd, width: int, height: int, diffuse: Texture | None = None,
               normal: Texture | None = None, shadow_size: int = 0, clear=((0, 0, 0, 255), _FLT_MAX),
               shadow_clear=((0, 0, 0, 255), _FLT_MAX), out: dict | None = None) -> int:
        """`out` may hold "color" (h,w,4) u8, "depth" (h,w) f32 and "prim" (h,w) u32 arrays
        (page-locked ones keep the copies asynchronous); they stay referenced until the
        request is waited for."""
        out = out or {}
        r = Request()
        r.mesh = mesh.handle
        r.shader = shader
        r.diffuse = diffuse.handle if diffuse else 0
        r.normal = normal.handle if normal else 0
        r.width, r.height, r.shadow_size = width, height, shadow_size
        sdb = np.ascontiguousarray(np.asarray(sd, dtype=SHADER_DATA_DTYPE).reshape(()))
        ctypes.memmove(ctypes.addressof(r.uniforms), sdb.ctypes.data, SHADER_DATA_DTYPE.itemsize)
        for i in range(4):
            r.clear_rgba[i] = clear[0][i]
            r.shadow_clear_rgba[i] = shadow_clear[0][i]
        r.clear_depth = float(clear[1])
        r.shadow_clear_depth = float(shadow_clear[1])
        arrays = []
        for key, field, dt, shape in (("color", "out_rgba", np.uint8, (height, width, 4)),
                                      ("depth", "out_depth", np.float32, (height, width)),
                                      ("prim", "out_prim", np.uint32, (height, width))):
            a = out.get(key)
            if a is not None:
                if a.dtype != dt or a.shape != shape or not a.flags.c_contiguous or not a.flags.writeable:
                    raise ValueError(f"out[{key!r}] must be a writeable contiguous {np.dtype(dt).name} {shape}")
                setattr(r, field, a.ctypes.data)
                arrays.append(a)
        t = ctypes.c_uint64()
        check(lib().hsr_server_submit(self.handle, ctypes.byref(r), ctypes.byref(t)))
        self._live[t.value] = tuple(arrays)
        return t.value

    @staticmethod
    def _status(st: RequestStatus) -> dict:
        return {k: getattr(st, k) for k, _ in RequestStatus._fields_}

    def inject_alloc_failures(self, n: int) -> None:
        """The next n target allocations fail as if the memory pool were exhausted."""
        check(lib().hsr_server_inject_alloc_failures(self.handle, n))

    def poll(self, ticket: int) -> dict | None:
        st = RequestStatus()
        rc = lib().hsr_server_poll(self.handle, ticket, ctypes.byref(st))
        if rc == ERR_BUSY:
            return None
        check(rc)
        self._live.pop(ticket, None)
        return self._status(st)

    def wait(self, ticket: int, timeout_ms: int = 120000) -> dict:
        st = RequestStatus()
        check(lib().hsr_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(st)))
        self._live.pop(ticket, None)
        return self._status(st)

    def now_ms(self) -> float:
        v = ctypes.c_double()
        check(lib().hsr_server_now_ms(self.handle, ctypes.byref(v)))
        return v.value

    def close(self) -> None:
        if self.handle:
            check(lib().hsr_server_destroy(self.handle))
            self.handle = 0
            self._live.clear()
