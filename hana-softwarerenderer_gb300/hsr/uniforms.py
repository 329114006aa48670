"""Host-side uniform builder: ShaderData the way DrawModel::draw fills it.

Every value is computed with IEEE float32 scalar operations in the reference's own
operation order, so the bits equal what the reference computes on the same host:

- ``lookat`` / ``perspective`` / ``orthographic``: maths.cpp:206-255
- matrix product: ``result[i][j] = lhs[i] * rhs.getCol(j)``, a dot product accumulated
  from the last index down (matrix.h:118-123, vector.h:69-73)
- ``invert``: cofactor adjugate / first-row dot / transpose (matrix.h:27-109)
- ``normalize``: ``v * (1 / sqrt(x*x + y*y + z*z))`` (vector.h:41-42)
- ``TO_RADIANS`` with ``PI = 3.1415927f`` (maths.h:6-9)
- camera constants FOVY 60 deg, NEAR 0.1, FAR 10000 (camera.cpp:11-14)
- ``light_vp = orthographic(aspect, 1, 0, 5) * lookat(light, target, up)`` (scene.h:69)
- ambient / light colour constants (scene.h:8-9), material defaults (scene.cpp:81-84)

``tan`` is the C library's ``tanf`` (the float overload the reference resolves to), called
through ctypes so the result matches the host's own ``tanf``.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

F32 = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.tanf.restype = ctypes.c_float
_libm.tanf.argtypes = [ctypes.c_float]

SHADER_DATA_DTYPE = np.dtype([
    ("view_pos", "<f4", 3),
    ("light_dir", "<f4", 3),
    ("light_color", "<f4", 4),
    ("ambient", "<f4", 4),
    ("model_matrix", "<f4", 16),
    ("model_matrix_I", "<f4", 16),
    ("view_matrix", "<f4", 16),
    ("projection_matrix", "<f4", 16),
    ("light_vp_matrix", "<f4", 16),
    ("camera_vp_matrix", "<f4", 16),
    ("enable_shadow", "<i4"),
    ("material_color", "<f4", 4),
    ("material_specular", "<f4", 4),
    ("gloss", "<f4"),
    ("bump_scale", "<f4"),
])
assert SHADER_DATA_DTYPE.itemsize == 484

PI = F32(3.1415927)
EPSILON = F32(1e-5)


def to_radians(deg) -> np.float32:
    return (PI / F32(180)) * F32(deg)


FOVY = to_radians(60)          # camera.cpp:13
NEAR = F32(0.1)                # camera.cpp:11
FAR = F32(10000)               # camera.cpp:12
UP = (F32(0), F32(1), F32(0))  # camera.cpp:14
ORIGIN = (F32(0), F32(0), F32(0))  # Camera::get_target_position (camera.cpp:94-97)

AMBIENT = (F32(54) / F32(255), F32(58) / F32(255), F32(66) / F32(255), F32(255))        # scene.h:8
LIGHT_COLOR = (F32(255) / F32(255), F32(244) / F32(255), F32(214) / F32(255), F32(255))  # scene.h:9
WHITE = (F32(1), F32(1), F32(1), F32(255))                                           # color.cpp:12
LIGHT_POS = (F32(2), F32(2), F32(2))                                                 # scene.cpp:7


def v3(x) -> tuple:
    return (F32(x[0]), F32(x[1]), F32(x[2]))


def sub3(a, b):
    return (F32(a[0] - b[0]), F32(a[1] - b[1]), F32(a[2] - b[2]))


def dot_rev(a, b) -> np.float32:
    """Vector operator* (vector.h:69-73): ret = 0; for i = N-1 .. 0: ret += a[i]*b[i]."""
    r = F32(0)
    for i in range(len(a) - 1, -1, -1):
        r = F32(r + F32(a[i] * b[i]))
    return r


def cross3(a, b):
    return (F32(a[1] * b[2] - a[2] * b[1]), F32(a[2] * b[0] - a[0] * b[2]), F32(a[0] * b[1] - a[1] * b[0]))


def normalize3(v):
    n = np.sqrt(F32(F32(F32(v[0] * v[0]) + F32(v[1] * v[1])) + F32(v[2] * v[2])))
    f = F32(F32(1) / F32(n))
    return (F32(v[0] * f), F32(v[1] * f), F32(v[2] * f))


class Mat4:
    """Matrix4x4 as a list of 4 row tuples of float32."""

    def __init__(self, rows):
        self.r = [list(map(F32, row)) for row in rows]

    @staticmethod
    def identity():
        return Mat4([[F32(1.0 if i == j else 0.0) for j in range(4)] for i in range(4)])

    def col(self, j):
        return [self.r[i][j] for i in range(len(self.r))]

    def __matmul__(self, o: "Mat4") -> "Mat4":
        rows = [[dot_rev(self.r[i], o.col(j)) for j in range(len(o.r[0]))] for i in range(len(self.r))]
        return Mat4(rows)

    def flat(self) -> np.ndarray:
        return np.array([x for row in self.r for x in row], dtype=np.float32)

    # --- invert (matrix.h:72-109) -------------------------------------------------
    @staticmethod
    def _det(m):
        n = len(m)
        if n == 1:
            return m[0][0]
        ret = F32(0)
        for i in range(n - 1, -1, -1):
            ret = F32(ret + F32(m[0][i] * Mat4._cofactor(m, 0, i)))
        return ret

    @staticmethod
    def _minor(m, row, col):
        n = len(m)
        return [[m[i if i < row else i + 1][j if j < col else j + 1] for j in range(n - 1)] for i in range(n - 1)]

    @staticmethod
    def _cofactor(m, row, col):
        sign = F32(-1) if (row + col) % 2 else F32(1)
        return F32(Mat4._det(Mat4._minor(m, row, col)) * sign)

    def invert(self) -> "Mat4":
        m = self.r
        adj = [[Mat4._cofactor(m, i, j) for j in range(4)] for i in range(4)]
        tmp = dot_rev(adj[0], m[0])
        it = [[F32(adj[i][j] / tmp) for j in range(4)] for i in range(4)]
        return Mat4([[it[j][i] for j in range(4)] for i in range(4)])


def lookat(eye, target, up) -> Mat4:
    z = normalize3(sub3(eye, target))
    x = normalize3(cross3(up, z))
    y = cross3(z, x)
    m = Mat4.identity()
    m.r[0] = [x[0], x[1], x[2], F32(0)]
    m.r[1] = [y[0], y[1], y[2], F32(0)]
    m.r[2] = [z[0], z[1], z[2], F32(0)]
    m.r[0][3] = F32(-dot_rev(x, eye))
    m.r[1][3] = F32(-dot_rev(y, eye))
    m.r[2][3] = F32(-dot_rev(z, eye))
    return m


def perspective(fovy, aspect, near, far) -> Mat4:
    fovy, aspect, near, far = F32(fovy), F32(aspect), F32(near), F32(far)
    z_range = F32(far - near)
    m = Mat4.identity()
    m.r[1][1] = F32(F32(1) / F32(_libm.tanf(float(F32(fovy / F32(2))))))
    m.r[0][0] = F32(m.r[1][1] / aspect)
    m.r[2][2] = F32(F32(-F32(near + far)) / z_range)
    m.r[2][3] = F32(F32(F32(F32(-2) * near) * far) / z_range)
    m.r[3][2] = F32(-1)
    m.r[3][3] = F32(0)
    return m


def orthographic(right, top, near, far) -> Mat4:
    right, top, near, far = F32(right), F32(top), F32(near), F32(far)
    z_range = F32(far - near)
    m = Mat4.identity()
    m.r[0][0] = F32(F32(1) / right)
    m.r[1][1] = F32(F32(1) / top)
    m.r[2][2] = F32(F32(-2) / z_range)
    m.r[2][3] = F32(F32(-F32(near + far)) / z_range)
    return m


_IDENTITY_INV = None


def shader_data(eye, width: int, height: int, *, target=(0, 0, 0), light=LIGHT_POS,
                model: Mat4 | None = None, enable_shadow: bool = False,
                material_color=WHITE, material_specular=WHITE, gloss=50.0, bump_scale=1.0,
                identity_mvp: bool = False) -> np.ndarray:
    """Fill one ShaderData record as DrawModel::draw does (scene.h:55-71).

    ``identity_mvp`` makes every matrix the identity (clip = (x, y, z, 1)), the setting of
    the depth-order stress workload.
    """
    global _IDENTITY_INV
    eye, target, light = v3(eye), v3(target), v3(light)
    sd = np.zeros((), dtype=SHADER_DATA_DTYPE)
    aspect = F32(F32(width) / F32(height))
    if identity_mvp:
        ident = Mat4.identity()
        model = view = proj = lvp = cvp = ident
        model_I = ident
    else:
        view = lookat(eye, target, UP)
        proj = perspective(FOVY, aspect, NEAR, FAR)
        if model is None:  # the identity's inverse (same routine, computed once)
            model = Mat4.identity()
            if _IDENTITY_INV is None:
                _IDENTITY_INV = model.invert()
            model_I = _IDENTITY_INV
        else:
            model_I = model.invert()
        # the light looks at Camera::get_target_position(), which returns the origin whatever
        # the camera's target (camera.cpp:94-97)
        lvp = orthographic(aspect, 1, 0, 5) @ lookat(light, ORIGIN, UP)
        cvp = proj @ view
    sd["view_pos"] = eye
    sd["light_dir"] = normalize3(sub3(light, ORIGIN))
    sd["light_color"] = LIGHT_COLOR
    sd["ambient"] = AMBIENT
    sd["model_matrix"] = model.flat()
    sd["model_matrix_I"] = model_I.flat()
    sd["view_matrix"] = view.flat()
    sd["projection_matrix"] = proj.flat()
    sd["light_vp_matrix"] = lvp.flat()
    sd["camera_vp_matrix"] = cvp.flat()
    sd["enable_shadow"] = 1 if enable_shadow else 0
    sd["material_color"] = material_color
    sd["material_specular"] = material_specular
    sd["gloss"] = F32(gloss)
    sd["bump_scale"] = F32(bump_scale)
    return sd
