"""CPU: the seeded workload generators for batched views and serving (host logic only)."""
import math

import numpy as np

from hsr import scenes

TINY_POOL = (("grid", 8), ("sphere", 2))


def test_pool_meshes_have_fixed_point_normals_and_sizes():
    pool = scenes.mesh_pool(TINY_POOL, seed=1)
    assert [p.mesh.nfaces for p in pool] == [2 * 8 * 8, 20 * 4 ** 2]
    for p in pool:
        n = p.mesh.nrm
        assert np.array_equal(scenes.ref_normalize(n).view(np.uint32), n.view(np.uint32))
        assert p.mesh.faces.max() < len(p.mesh.pos)


def test_pool_specs_match_workload_sizes():
    tris = lambda kind, s: 20 * 4 ** s if kind == "sphere" else 2 * s * s  # noqa: E731
    view = [tris(k, s) for k, s in scenes.VIEW_POOL_SPEC]
    assert len(view) == 8 and min(view) == 2048 and max(view) == 1310720
    serve = [tris(k, s) for k, s in scenes.SERVE_POOL_SPEC]
    assert len(serve) == 16 and 7.5e6 < sum(serve) < 8.5e6


def test_view_set_distribution():
    pool = scenes.mesh_pool(TINY_POOL, seed=1)
    views = scenes.view_set(pool, n=64, seed=3)
    assert len(views) == 64
    assert {(v.width, v.height) for v in views} <= {(256, 256), (512, 512), (1280, 720), (1920, 1080)}
    assert {v.shader for v in views} == {scenes.BLINN, scenes.NORMALMAP}
    assert {v.shadow for v in views} == {0, 2048}
    for v in views:  # the uniforms carry the view's own aspect and shadow flag
        assert int(v.sd["enable_shadow"]) == (1 if v.shadow else 0)
    again = scenes.view_set(pool, n=64, seed=3)
    assert all(a.sd.tobytes() == b.sd.tobytes() for a, b in zip(views, again))


def test_request_stream_is_poisson_and_log_uniform():
    pool = scenes.mesh_pool(TINY_POOL, seed=1)
    reqs = scenes.request_stream(pool, 400, rate_per_s=1000.0, seed=5)
    t = np.array([r.arrival_ms for r in reqs])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    gap = np.diff(t).mean()
    assert 0.8 < gap < 1.2  # 1 ms mean gap at 1000 requests/s
    w = np.array([r.width for r in reqs])
    h = np.array([r.height for r in reqs])
    assert w.min() >= 128 and w.max() <= 3840 and h.min() >= 128 and h.max() <= 2160
    # log-uniform: about half the widths below the geometric midpoint
    assert 0.4 < np.mean(w < math.sqrt(128 * 3840)) < 0.6
    assert set(r.shader for r in reqs) == set(scenes.REQUEST_SHADERS)
    sh = [r.shadow for r in reqs if r.shadow]
    assert 0.4 < len(sh) / len(reqs) < 0.6
    assert all(s in (256, 512, 1024, 2048) and s >= min(2048, max(r.width, r.height))
               for r in reqs for s in [r.shadow] if s)


def test_retime_keeps_requests():
    pool = scenes.mesh_pool(TINY_POOL, seed=1)
    reqs = scenes.request_stream(pool, 50, rate_per_s=100.0, seed=5)
    fast = scenes.retime(reqs, 10000.0)
    assert [(r.mesh, r.width, r.height, r.shader, r.shadow) for r in reqs] == \
        [(r.mesh, r.width, r.height, r.shader, r.shadow) for r in fast]
    assert fast[-1].arrival_ms < reqs[-1].arrival_ms


def test_view_frame_matches_request():
    pool = scenes.mesh_pool(TINY_POOL, seed=1)
    tex = scenes.pool_textures(2, 16, seed=2)
    r = scenes.request_stream(pool, 3, rate_per_s=10.0, seed=8)[1]
    f = scenes.view_frame(r, pool, tex)
    assert (f.width, f.height, f.shader) == (r.width, r.height, r.shader)
    assert f.shadow_size == (r.shadow, r.shadow)
    assert f.mesh is pool[r.mesh].mesh
