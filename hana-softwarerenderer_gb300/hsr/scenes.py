"""Seeded synthetic workloads for the draw path (no public dataset is involved).

Every workload is generated from a seed with numpy's PCG64, so it can be rebuilt on any
host.  Normals are forced to fixed points of the reference's ``Vector3f::normalize``
(vector.h:41-42): ``Model::normal()`` normalises the stored normal in place on every
access (model.cpp:108-111), and only for fixed points is that mutation a no-op, which
keeps a frame independent of how many times it was drawn before.

Workloads (sizes as named in the benchmark description):

- ``sphere_frame``: icosphere of a given subdivision, radius 1, smooth normals,
  spherical uvs, uniform-noise RGBA8 diffuse; Blinn-Phong, camera at distance 3.
  Subdivision 4 at 512x512 is the plain CPU-runnable frame.
- ``displaced_frame``: icosphere subdivision 7 with fractal radial displacement
  (amplitude 0.05) and a 2-triangle ground plane submitted after it; 1024^2 diffuse +
  tangent-space normal map; 1920x1080 with a 2048^2 shadow map; NormalMap + shadow.
- ``soup_frame``: triangle soup with identity transforms (clip = (x, y, z, 1)),
  centroids uniform on screen, lognormal edge lengths, constant per-triangle NDC depth,
  1% exact duplicates submitted later (equal-depth ties); flat test shader.
- ``view_pool`` / ``request_stream``: meshes, cameras and requests for batched views
  and the serving loop.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

from . import uniforms as U

F32 = np.float32

# hsr_shader_kind (include/hsr.h)
GROUND, TOON, TEXTURE, TEXTURE_WITH_LIGHT, BLINN, NORMALMAP, SHADOW, FLAT = range(8)
SHADER_NAMES = ["ground", "toon", "texture", "texture_with_light", "blinn", "normalmap", "shadow", "flat"]

FLT_MAX = float(np.finfo(np.float32).max)


@dataclasses.dataclass
class Mesh:
    pos: np.ndarray    # (npos, 3) float32
    nrm: np.ndarray    # (nnrm, 3) float32
    uv: np.ndarray     # (nuv, 2) float32
    faces: np.ndarray  # (nfaces, 3, 3) int32: corner -> (v, vt, vn), 0-based

    @property
    def nfaces(self) -> int:
        return int(self.faces.shape[0])

    def nbytes(self) -> int:
        return self.pos.nbytes + self.nrm.nbytes + self.uv.nbytes + self.faces.nbytes


@dataclasses.dataclass
class Texture:
    data: np.ndarray   # (h, w, bpp) uint8, TGAImage layout: texel (x, y) = data[y, x], bytes B,G,R(,A)

    @property
    def w(self) -> int:
        return int(self.data.shape[1])

    @property
    def h(self) -> int:
        return int(self.data.shape[0])

    @property
    def bpp(self) -> int:
        return int(self.data.shape[2])


@dataclasses.dataclass
class Frame:
    """One DrawModel::draw (scene.h:53-99): optional shadow pass, then the main pass."""
    mesh: Mesh
    shader: int
    sd: np.ndarray                      # SHADER_DATA_DTYPE record
    width: int
    height: int
    diffuse: Optional[Texture] = None
    normal: Optional[Texture] = None
    shadow_size: tuple = (0, 0)         # (0, 0): no shadow pass
    clear_rgba: tuple = (0, 0, 0, 1)    # per-frame clear of main.cpp:152 (Black -> alpha byte 1 on x86)
    clear_depth: float = FLT_MAX        # main.cpp:153
    shadow_clear_rgba: tuple = (0, 0, 0, 1)  # scene.h:96
    shadow_clear_depth: float = FLT_MAX      # scene.h:97
    name: str = ""


# ---------------------------------------------------------------------------------
# reference-arithmetic helpers (vectorised float32)
# ---------------------------------------------------------------------------------
def ref_normalize(v: np.ndarray) -> np.ndarray:
    """Vector3f::normalize on rows: v * (1 / sqrt(x*x + y*y + z*z)), float32 ops."""
    v = v.astype(np.float32, copy=False)
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    n = np.sqrt((x * x + y * y) + z * z)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.float32(1) / n
    return np.stack([x * f, y * f, z * f], axis=1).astype(np.float32)


def _is_fixed(n: np.ndarray) -> np.ndarray:
    return (ref_normalize(n).view(np.uint32) == n.view(np.uint32)).all(axis=1)


def fixed_point_normals(n: np.ndarray, max_tries: int = 200) -> np.ndarray:
    """Replace each row by a nearby bitwise fixed point of ref_normalize.

    Rows that land in a 2-cycle are nudged by a few ulps in one component (deterministic
    sequence of nudges) and normalised again until they settle on a fixed point."""
    base = ref_normalize(np.asarray(n, dtype=np.float32))
    base = ref_normalize(base)
    out = base.copy()
    bad = ~_is_fixed(out)
    k = 0
    while bad.any():
        if k >= max_tries:
            raise RuntimeError("normals did not reach fixed points")
        comp, steps = k % 3, 1 + k // 3
        cand = base[bad].copy()
        c = cand[:, comp].view(np.int32).astype(np.int64)
        c += steps if (k // 3) % 2 == 0 else -steps
        cand[:, comp] = c.astype(np.int32).view(np.float32)
        cand = ref_normalize(ref_normalize(cand))
        ok = _is_fixed(cand)
        idx = np.nonzero(bad)[0]
        out[idx[ok]] = cand[ok]
        bad[idx[ok]] = False
        k += 1
    return out


# ---------------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------------
def icosphere(subdiv: int):
    """Unit icosphere: (positions float64 (n,3), faces int64 (m,3)), CCW seen from outside."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key[:, 0] * (len(v) + 1) + key[:, 1], return_inverse=True)
        e0 = uniq // (len(v) + 1)
        e1 = uniq % (len(v) + 1)
        mid = v[e0] + v[e1]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        m = inv.reshape(3, -1) + base
        ab, bc, ca = m[0], m[1], m[2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return v, f


def spherical_uv(p: np.ndarray) -> np.ndarray:
    u = 0.5 + np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi)
    w = 0.5 - np.arcsin(np.clip(p[:, 1], -1, 1)) / np.pi
    return np.stack([u, w], 1).astype(np.float32)


def fbm(p: np.ndarray, seed: int, octaves: int = 5) -> np.ndarray:
    """Fractal sum of seeded sinusoidal plane waves, roughly in [-1, 1]."""
    rng = np.random.default_rng(seed)
    out = np.zeros(len(p))
    amp, freq, norm = 1.0, 2.0, 0.0
    for _ in range(octaves):
        d = rng.normal(size=(6, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        ph = rng.uniform(0, 2 * np.pi, size=6)
        out += amp * np.sin(freq * (p @ d.T) + ph).sum(axis=1) / math.sqrt(6)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def smooth_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    p = pos.astype(np.float64)
    fn = np.cross(p[faces[:, 1]] - p[faces[:, 0]], p[faces[:, 2]] - p[faces[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n


def indexed_mesh(pos, nrm, uv, tri) -> Mesh:
    """Mesh whose v, vt and vn indices are all the triangle's vertex indices."""
    tri = np.asarray(tri, dtype=np.int32)
    faces = np.repeat(tri[:, :, None], 3, axis=2).astype(np.int32)
    return Mesh(np.ascontiguousarray(pos, np.float32), fixed_point_normals(nrm),
                np.ascontiguousarray(uv, np.float32), np.ascontiguousarray(faces))


def concat_meshes(a: Mesh, b: Mesh) -> Mesh:
    """b's faces are submitted after a's (sequence order continues)."""
    off = np.array([len(a.pos), len(a.uv), len(a.nrm)], dtype=np.int32)
    return Mesh(np.concatenate([a.pos, b.pos]), np.concatenate([a.nrm, b.nrm]),
                np.concatenate([a.uv, b.uv]), np.concatenate([a.faces, b.faces + off[None, None, :]]))


def ground_plane(y: float, extent: float) -> Mesh:
    pos = np.array([[-extent, y, -extent], [extent, y, -extent], [extent, y, extent], [-extent, y, extent]], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    nrm = np.array([[0, 1, 0]] * 4, np.float32)
    tri = np.array([[0, 2, 1], [0, 3, 2]], np.int32)   # CCW seen from +y
    return indexed_mesh(pos, nrm, uv, tri)


def noise_texture(w: int, h: int, bpp: int, seed: int) -> Texture:
    rng = np.random.default_rng(seed)
    return Texture(rng.integers(0, 256, size=(h, w, bpp), dtype=np.uint8))


def normal_map_texture(w: int, h: int, seed: int, spread: int = 40) -> Texture:
    """24-bit tangent-space normal map, bytes B,G,R with (R,G,B) around (128,128,255)."""
    rng = np.random.default_rng(seed)
    d = np.empty((h, w, 3), np.uint8)
    d[:, :, 0] = 255 - rng.integers(0, spread, size=(h, w))          # B -> z
    d[:, :, 1] = 128 + rng.integers(-spread, spread + 1, size=(h, w))  # G -> y
    d[:, :, 2] = 128 + rng.integers(-spread, spread + 1, size=(h, w))  # R -> x
    return Texture(d)


def sphere_mesh(subdiv: int, displace: float = 0.0, seed: int = 0) -> Mesh:
    p, f = icosphere(subdiv)
    if displace:
        r = 1.0 + displace * fbm(p, seed)
        pd = p * r[:, None]
        n = smooth_normals(pd, f)
    else:
        pd, n = p, p
    return indexed_mesh(pd.astype(np.float32), n.astype(np.float32), spherical_uv(p), f)


def grid_mesh(nx: int, nz: int, seed: int, amp: float = 0.15) -> Mesh:
    """Height-field grid over [-1,1]^2 (2*nx*nz triangles)."""
    xs = np.linspace(-1, 1, nx + 1)
    zs = np.linspace(-1, 1, nz + 1)
    X, Z = np.meshgrid(xs, zs)
    P = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], 1)
    P[:, 1] = amp * fbm(P, seed)
    idx = np.arange((nx + 1) * (nz + 1)).reshape(nz + 1, nx + 1)
    a, b = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
    c, d = idx[1:, 1:].ravel(), idx[1:, :-1].ravel()
    tri = np.concatenate([np.stack([a, d, c], 1), np.stack([a, c, b], 1)])  # CCW from +y
    n = smooth_normals(P, tri)
    uv = np.stack([(X.ravel() + 1) / 2, (Z.ravel() + 1) / 2], 1)
    return indexed_mesh(P.astype(np.float32), n.astype(np.float32), uv.astype(np.float32), tri)


# ---------------------------------------------------------------------------------
# frames
# ---------------------------------------------------------------------------------
def sphere_frame(subdiv: int = 4, width: int = 512, height: int = 512, shader: int = BLINN,
                 eye=(0.0, 0.0, 3.0), tex_size: int = 256, seed: int = 1, shadow: int = 0,
                 nm_size: int = 0) -> Frame:
    mesh = sphere_mesh(subdiv)
    sd = U.shader_data(eye, width, height, enable_shadow=bool(shadow))
    nm = normal_map_texture(nm_size, nm_size, seed + 1) if nm_size else None
    return Frame(mesh, shader, sd, width, height, diffuse=noise_texture(tex_size, tex_size, 4, seed),
                 normal=nm, shadow_size=(shadow, shadow) if shadow else (0, 0),
                 name=f"sphere{subdiv}_{width}x{height}_{SHADER_NAMES[shader]}")


def displaced_frame(subdiv: int = 7, width: int = 1920, height: int = 1080, shadow: int = 2048,
                    tex_size: int = 1024, shader: int = NORMALMAP, seed: int = 7,
                    eye=(0.0, 0.8, 3.2), plane_extent: float = 6.0) -> Frame:
    mesh = concat_meshes(sphere_mesh(subdiv, displace=0.05, seed=seed), ground_plane(-1.2, plane_extent))
    sd = U.shader_data(eye, width, height, enable_shadow=bool(shadow))
    return Frame(mesh, shader, sd, width, height, diffuse=noise_texture(tex_size, tex_size, 4, seed + 1),
                 normal=normal_map_texture(tex_size, tex_size, seed + 2),
                 shadow_size=(shadow, shadow) if shadow else (0, 0),
                 name=f"displaced{subdiv}_{width}x{height}_{SHADER_NAMES[shader]}_shadow{shadow}")


def soup_frame(ntri: int = 4_000_000, width: int = 3840, height: int = 2160, seed: int = 11,
               median_edge_px: float = 2.0, sigma: float = 1.06, dup_frac: float = 0.01) -> Frame:
    """Depth-order stress: CCW triangles in NDC with constant depth, plus exact duplicates."""
    rng = np.random.default_rng(seed)
    nbase = ntri - int(round(ntri * dup_frac))
    cx = rng.uniform(0, width, nbase)
    cy = rng.uniform(0, height, nbase)
    edge = median_edge_px * np.exp(sigma * rng.standard_normal(nbase))
    r = edge / math.sqrt(3.0)
    th = rng.uniform(0, 2 * np.pi, nbase)[:, None] + np.array([0, 2 * np.pi / 3, 4 * np.pi / 3])[None, :]
    th = th + rng.uniform(-0.35, 0.35, (nbase, 3))
    px = cx[:, None] + r[:, None] * np.cos(th)
    py = cy[:, None] + r[:, None] * np.sin(th)
    z = rng.uniform(0, 1, nbase)
    pos = np.empty((nbase, 3, 3), np.float32)
    pos[:, :, 0] = (px / width * 2 - 1).astype(np.float32)
    pos[:, :, 1] = (py / height * 2 - 1).astype(np.float32)
    pos[:, :, 2] = z.astype(np.float32)[:, None]
    pos = pos.reshape(-1, 3)
    tri = np.arange(nbase * 3, dtype=np.int64).reshape(nbase, 3)
    ndup = ntri - nbase
    if ndup:
        src = np.sort(rng.choice(nbase, ndup, replace=False))
        # each duplicate is inserted at a random later position (same vertices -> equal depth)
        order = np.arange(nbase, dtype=np.int64)
        ins = rng.integers(0, nbase + 1, ndup)
        ins = np.maximum(ins, src + 1)
        allf = np.concatenate([order, src])
        key = np.concatenate([order.astype(np.float64), ins - 0.5])
        tri = tri[allf[np.argsort(key, kind="stable")]]
    faces = np.zeros((ntri, 3, 3), np.int32)
    faces[:, :, 0] = tri
    mesh = Mesh(pos, np.array([[0, 0, 1]], np.float32), np.zeros((1, 2), np.float32), faces)
    sd = U.shader_data((0, 0, 1), width, height, identity_mvp=True)
    return Frame(mesh, FLAT, sd, width, height, name=f"soup{ntri}_{width}x{height}")


# ---------------------------------------------------------------------------------
# batched views and serving
# ---------------------------------------------------------------------------------
# hsr_shader_kind values a request may ask for (the reference scenes' shaders)
REQUEST_SHADERS = (GROUND, TOON, TEXTURE, TEXTURE_WITH_LIGHT, BLINN, NORMALMAP)


@dataclasses.dataclass
class PoolMesh:
    mesh: Mesh
    kind: str          # "sphere" | "grid"
    name: str


def pool_mesh(kind: str, size: int, seed: int) -> PoolMesh:
    """A displaced icosphere of subdivision `size` (20*4^size triangles) or a height-field
    grid of size x size cells (2*size^2 triangles)."""
    if kind == "sphere":
        return PoolMesh(sphere_mesh(size, displace=0.05, seed=seed), kind, f"ico{size}_s{seed}")
    return PoolMesh(grid_mesh(size, size, seed), kind, f"grid{size}_s{seed}")


# 8 meshes from 2,048 to 1,310,720 triangles (roughly geometric)
VIEW_POOL_SPEC = (("grid", 32), ("sphere", 4), ("sphere", 5), ("grid", 128),
                  ("sphere", 6), ("grid", 256), ("sphere", 7), ("sphere", 8))
# 16 meshes, 8,257,536 triangles in total
SERVE_POOL_SPEC = (("sphere", 8),) * 3 + (("sphere", 7),) * 6 + (("grid", 512),) * 4 + (("sphere", 6),) * 3


def mesh_pool(spec, seed: int) -> list:
    return [pool_mesh(kind, size, seed + 101 * i) for i, (kind, size) in enumerate(spec)]


def orbit_eye(rng: np.random.Generator, kind: str) -> tuple:
    """Random orbit camera around the origin at radius 2-4; grids are seen from above
    (their triangles face +y)."""
    r = rng.uniform(2.0, 4.0)
    az = rng.uniform(0, 2 * np.pi)
    el = rng.uniform(0.35, 1.1) if kind == "grid" else rng.uniform(-0.6, 1.0)
    return (float(r * math.cos(el) * math.sin(az)), float(r * math.sin(el)), float(r * math.cos(el) * math.cos(az)))


@dataclasses.dataclass
class View:
    """One DrawModel::draw on a pooled mesh: which mesh / textures, target size, shader,
    uniforms and shadow map size (0: no shadow pass)."""
    mesh: int
    tex: int
    shader: int
    width: int
    height: int
    shadow: int
    sd: np.ndarray


def view_set(pool: list, n: int = 64, seed: int = 3, ntex: int = 4) -> list:
    """64 views: resolution uniform over {256^2, 512^2, 1280x720, 1920x1080}, mesh uniform
    over the pool, 50/50 Blinn / NormalMap, shadow pass (2048^2) on half of them."""
    rng = np.random.default_rng(seed)
    res = ((256, 256), (512, 512), (1280, 720), (1920, 1080))
    out = []
    for _ in range(n):
        m = int(rng.integers(len(pool)))
        w, h = res[int(rng.integers(4))]
        shader = BLINN if rng.random() < 0.5 else NORMALMAP
        shadow = 2048 if rng.random() < 0.5 else 0
        eye = orbit_eye(rng, pool[m].kind)
        sd = U.shader_data(eye, w, h, enable_shadow=bool(shadow))
        out.append(View(m, int(rng.integers(ntex)), shader, w, h, shadow, sd))
    return out


def serve_shadow_size(w: int, h: int) -> int:
    """Square shadow map for a w x h request: the next power of two of the larger side,
    clamped to [256, 2048]."""
    s = 256
    while s < max(w, h) and s < 2048:
        s *= 2
    return s


@dataclasses.dataclass
class Request(View):
    arrival_ms: float = 0.0


def request_stream(pool: list, n: int, rate_per_s: float, seed: int = 5, ntex: int = 4) -> list:
    """Poisson arrivals at `rate_per_s`; mesh uniform from the pool; width and height
    log-uniform over [128, 3840] x [128, 2160]; shader uniform over REQUEST_SHADERS; shadow
    pass on half of the requests."""
    rng = np.random.default_rng(seed)
    gaps = np.random.default_rng(seed + 7919).exponential(1000.0 / rate_per_s, n)
    t = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n):  # request i does not depend on n or on the rate
        m = int(rng.integers(len(pool)))
        w = int(round(math.exp(rng.uniform(math.log(128), math.log(3840)))))
        h = int(round(math.exp(rng.uniform(math.log(128), math.log(2160)))))
        shader = int(REQUEST_SHADERS[int(rng.integers(len(REQUEST_SHADERS)))])
        shadow = serve_shadow_size(w, h) if rng.random() < 0.5 else 0
        eye = orbit_eye(rng, pool[m].kind)
        sd = U.shader_data(eye, w, h, enable_shadow=bool(shadow))
        out.append(Request(m, int(rng.integers(ntex)), shader, w, h, shadow, sd, float(t[i])))
    return out


def retime(requests: list, rate_per_s: float, seed: int = 9) -> list:
    """The same requests with new Poisson arrival times."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1000.0 / rate_per_s, len(requests))
    t = np.cumsum(gaps) - gaps[0]
    return [dataclasses.replace(r, arrival_ms=float(ti)) for r, ti in zip(requests, t)]


def view_frame(v: View, pool: list, textures: list) -> Frame:
    """The Frame (oracle input) equal to a view / request."""
    d, nm = textures[v.tex]
    return Frame(pool[v.mesh].mesh, v.shader, v.sd, v.width, v.height, diffuse=d, normal=nm,
                 shadow_size=(v.shadow, v.shadow), clear_rgba=(0, 0, 0, 255), shadow_clear_rgba=(0, 0, 0, 255),
                 name=f"view_{pool[v.mesh].name}_{v.width}x{v.height}_{SHADER_NAMES[v.shader]}_sh{v.shadow}")


def pool_textures(n: int = 4, size: int = 1024, seed: int = 17) -> list:
    """n (diffuse RGBA8, tangent normal map RGB8) pairs of size^2."""
    return [(noise_texture(size, size, 4, seed + 2 * i), normal_map_texture(size, size, seed + 2 * i + 1))
            for i in range(n)]


def prim_id_mesh(mesh: Mesh) -> Mesh:
    """Same v / vn / faces, one vt per face carrying the face id (lo 12 bits, hi bits)."""
    nf = mesh.nfaces
    fid = np.arange(nf, dtype=np.int64)
    uv = np.stack([(fid & 4095).astype(np.float32), (fid >> 12).astype(np.float32)], 1)
    faces = mesh.faces.copy()
    faces[:, :, 1] = fid[:, None].astype(np.int32)
    return Mesh(mesh.pos, mesh.nrm, uv, faces)


def soup_depth_complexity(frame: Frame) -> float:
    p = frame.mesh.pos[frame.mesh.faces[:, :, 0]].astype(np.float64)
    x = (p[:, :, 0] + 1) * 0.5 * frame.width
    y = (p[:, :, 1] + 1) * 0.5 * frame.height
    area = 0.5 * np.abs((x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0]))
    return float(area.sum() / (frame.width * frame.height))


# ---------------------------------------------------------------------------------
# OBJ writer (exact float round trip: %.9g, read back by Model::Model, model.cpp:6-48)
# ---------------------------------------------------------------------------------
def write_obj(mesh: Mesh, path: str) -> None:
    with open(path, "w") as f:
        for p in mesh.pos.astype(np.float32):
            f.write("v %.9g %.9g %.9g\n" % (float(p[0]), float(p[1]), float(p[2])))
        for t in mesh.uv.astype(np.float32):
            f.write("vt  %.9g %.9g 0\n" % (float(t[0]), float(t[1])))
        for n in mesh.nrm.astype(np.float32):
            f.write("vn  %.9g %.9g %.9g\n" % (float(n[0]), float(n[1]), float(n[2])))
        fc = mesh.faces.astype(np.int64) + 1
        for c in fc:
            f.write("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % tuple(c.reshape(-1)))
