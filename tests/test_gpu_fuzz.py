"""GPU: randomized scenes against the oracle — every shader, with and without a shadow pass,
targets from 1x1 to 300x200 (sizes that are not multiples of the tile), triangle soups around
and behind the camera (faces through the near plane and the side planes go through the
clipper), triangles larger than a whole target (split into sub-records), degenerate and
back-facing triangles, unshared vertex / uv / normal indices, textures of 1, 3 and 4 bytes per
texel, and draws without the fused clear over random buffer contents.

Tolerances as in test_gpu_parity: depth, prim ids and alpha bit for bit, RGB within 1 LSB.
"""
import numpy as np
import pytest

import golden_io
import oracle
from hsr import scenes
from hsr import uniforms as U

pytestmark = pytest.mark.gpu

SHADERS = (scenes.GROUND, scenes.TOON, scenes.TEXTURE, scenes.TEXTURE_WITH_LIGHT, scenes.BLINN, scenes.NORMALMAP,
           scenes.SHADOW, scenes.FLAT)


def random_mesh(rng, nfaces: int) -> scenes.Mesh:
    """A soup around the origin: mostly small triangles, some huge, some degenerate, with
    independent v / vt / vn indices and unit normals that are fixed points of normalize."""
    npos, nuv, nnrm = 3 * nfaces // 2 + 3, nfaces + 3, nfaces // 2 + 3
    centers = rng.uniform(-2.5, 2.5, (npos, 3))
    pos = centers + rng.normal(0, 0.08, (npos, 3))
    big = rng.random(npos) < 0.01
    pos[big] *= rng.uniform(3, 20, (big.sum(), 1))  # far out: huge or clipped triangles
    uv = rng.uniform(-0.1, 1.1, (nuv, 2))  # a little outside [0, 1]: out-of-range texels read 0
    nrm = scenes.fixed_point_normals(rng.normal(0, 1, (nnrm, 3)))
    faces = np.empty((nfaces, 3, 3), np.int32)
    faces[:, :, 0] = rng.integers(0, npos, (nfaces, 3))
    # locality: most faces use three nearby vertices (small triangles)
    near = rng.random(nfaces) < 0.85
    base = rng.integers(0, npos - 3, nfaces)
    faces[near, :, 0] = base[near, None] + np.arange(3)[None, :]
    faces[:, :, 1] = rng.integers(0, nuv, (nfaces, 3))
    faces[:, :, 2] = rng.integers(0, nnrm, (nfaces, 3))
    degen = rng.random(nfaces) < 0.02
    faces[degen, 2, 0] = faces[degen, 1, 0]  # two equal corners
    return scenes.Mesh(pos.astype(np.float32), nrm, uv.astype(np.float32), faces)


def random_frame(seed: int) -> scenes.Frame:
    rng = np.random.default_rng(1000 + seed)
    w = int(rng.choice([1, 2, 7, 8, 9, 15, 16, 17, 63, 100, 161, 256, 300]))
    h = int(rng.choice([1, 3, 8, 16, 33, 64, 99, 128, 200]))
    shader = int(SHADERS[seed % len(SHADERS)])
    mesh = random_mesh(rng, int(rng.integers(1, 1500)))
    r = float(rng.uniform(0.5, 4.0))  # close cameras put faces behind the near plane
    th, ph = rng.uniform(0, 2 * np.pi), rng.uniform(0.2, 2.9)
    eye = (r * np.sin(ph) * np.cos(th), r * np.cos(ph), r * np.sin(ph) * np.sin(th))
    shadow = int(rng.choice([0, 0, 16, 64, 129])) if shader != scenes.SHADOW else 0
    sd = U.shader_data(eye, w, h, enable_shadow=bool(shadow), gloss=float(rng.uniform(1, 80)),
                       bump_scale=float(rng.uniform(0.2, 2.0)))
    bpp = int(rng.choice([1, 3, 4]))
    tex = scenes.noise_texture(int(rng.integers(1, 40)), int(rng.integers(1, 40)), bpp, seed)
    nm = scenes.normal_map_texture(int(rng.integers(1, 40)), int(rng.integers(1, 40)), seed + 7)
    return scenes.Frame(mesh, shader, sd, w, h, diffuse=tex, normal=nm,
                        shadow_size=(shadow, shadow) if shadow else (0, 0), name=f"fuzz{seed}")


def expect(frame):
    out = oracle.render_frame(frame)
    return {k: {"depth": v.depth, "color": v.color, "prim": v.prim} for k, v in out.items()}


def check(got, exp, label):
    for k in exp:
        golden_io.assert_pass(got[k], exp[k], k, label)


@pytest.mark.parametrize("seed", range(48))
def test_random_frame_vs_oracle(gpu, seed):
    from hsr import frame as hframe

    fr = random_frame(seed)
    g = hframe.GpuFrame(fr)
    try:
        g.render(batched=seed % 2 == 0)
        got = g.download()
    finally:
        g.release()
    check(got, expect(fr), fr.name)


@pytest.mark.parametrize("seed", range(8))
def test_random_draw_without_clear_vs_oracle(gpu, seed):
    """The draw reads the target's existing depth (and keeps its alpha) when not clearing."""
    import hsr

    fr = random_frame(100 + seed)
    rng = np.random.default_rng(seed)
    color = rng.integers(0, 256, (fr.height, fr.width, 4), dtype=np.uint8)
    depth = rng.uniform(0.2, 1.2, (fr.height, fr.width)).astype(np.float32)
    prim = rng.integers(0, 1 << 31, (fr.height, fr.width), dtype=np.uint32)
    prim_base = int(rng.integers(0, 1 << 20))
    tgt = hsr.Target(fr.width, fr.height)
    m, t, n = hsr.Mesh(fr.mesh), hsr.Texture(fr.diffuse), hsr.Texture(fr.normal)
    keep = []
    try:
        tgt.upload(color, depth, prim)
        hsr.draw(hsr.make_desc(m, fr.shader, fr.sd, tgt, t, n, prim_base=prim_base, keep=keep))
        got = tgt.download()
    finally:
        for o in (tgt, m, t, n):
            o.release()
    rb = oracle.Buffers(fr.width, fr.height)
    rb.color[:] = color
    rb.depth[:] = depth
    rb.prim[:] = prim
    oracle.draw(fr.mesh, fr.shader, fr.sd, rb, fr.diffuse, fr.normal, prim_base=prim_base)
    check({"main": got}, {"main": {"depth": rb.depth, "color": rb.color, "prim": rb.prim}}, f"noclear{seed}")
