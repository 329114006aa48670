"""GPU parity of the benchmark's own batches at their full size.

- The serving workload: 16 resident meshes (8,241,152 triangles), 1024^2 textures, requests
  with targets up to 3840x2160 and shadow maps up to 2048^2; the batch is requests 320-383 of
  the seed-5 stream, the first batch the benchmark times (after five warm-up batches).
- The 64-view workload: 8 meshes of 2,048-1,310,720 triangles, 256^2-1920x1080 targets,
  Blinn / NormalMap, 2048^2 shadow pass on half the views (view_set seed 3).

Each batch is drawn as one launch sequence.  Every view must equal the same view drawn
alone (all three planes bit for bit: a view's pixels do not depend on its batch), and the
largest views plus one view of every shader present must match the oracle: depth, prim ids
and alpha bit for bit, RGB within 1 LSB for the main pass (powf), bit for bit for the shadow
pass.  The oracle frames run on a thread pool (the oracle releases the GIL).
Reference: graphics_draw_triangle (graphics.cpp:378-407) called as DrawModel::draw does
(scene.h:73-99), IShader.cpp for the shaders.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import golden_io
import oracle
from hsr import scenes
from hsr import serve as hserve

pytestmark = pytest.mark.gpu

N_ORACLE_LARGEST = 8


def _pick_for_oracle(views):
    """The N largest views (main + shadow pixels), then one view of each shader not yet in."""
    size = [v.width * v.height + v.shadow * v.shadow for v in views]
    order = sorted(range(len(views)), key=lambda i: -size[i])
    pick = order[:N_ORACLE_LARGEST]
    have = {views[i].shader for i in pick}
    for i in order:
        if views[i].shader not in have:
            pick.append(i)
            have.add(views[i].shader)
    return pick


def _check_batch(rp, views, label):
    vb = hserve.ViewBatch(rp, views)
    try:
        vb.draw_all()
        got = []
        for i in range(len(views)):
            g = {"main": vb.mains[i].download()}
            if vb.shadows[i] is not None:
                g["shadow"] = vb.shadows[i].download()
            got.append(g)
    finally:
        vb.release()
    # every view equals itself drawn alone
    for i, v in enumerate(views):
        one = hserve.ViewBatch(rp, [v])
        try:
            one.draw_all()
            alone = {"main": one.mains[0].download()}
            if one.shadows[0] is not None:
                alone["shadow"] = one.shadows[0].download()
        finally:
            one.release()
        for k in alone:
            for p in ("color", "depth", "prim"):
                assert np.array_equal(got[i][k][p], alone[k][p]), (label, i, k, p)
    # the largest views and every shader against the oracle
    pick = _pick_for_oracle(views)
    frames = {i: scenes.view_frame(views[i], rp.pool, rp.tex_data) for i in pick}
    with cf.ThreadPoolExecutor(max_workers=min(len(pick), os.cpu_count() or 1)) as ex:
        exp = dict(zip(pick, ex.map(lambda i: oracle.render_frame(frames[i]), pick)))
    for i in pick:
        v = views[i]
        tag = f"{label} view {i} {v.width}x{v.height} {scenes.SHADER_NAMES[v.shader]} shadow {v.shadow}"
        for k, e in exp[i].items():
            golden_io.assert_pass(got[i][k], {"depth": e.depth, "color": e.color, "prim": e.prim}, k, tag)
    return pick


@pytest.fixture(scope="module")
def serve_pool(gpu):
    pool = scenes.mesh_pool(scenes.SERVE_POOL_SPEC, seed=1)
    tex = scenes.pool_textures(4, 1024, seed=17)
    rp = hserve.ResidentPool(pool, tex)
    rp.tex_data = tex
    yield rp
    rp.release()


def test_serving_batch_at_full_size(serve_pool):
    pool = serve_pool.pool
    assert sum(p.mesh.nfaces for p in pool) == 8_241_152
    reqs = scenes.request_stream(pool, 384, rate_per_s=1000.0, seed=5)[320:384]
    assert max(r.width * r.height for r in reqs) > 1920 * 1080  # some targets beyond 1080p
    assert max(r.shadow for r in reqs) == 2048
    pick = _check_batch(serve_pool, reqs, "serve batch")
    assert {reqs[i].shader for i in pick} == {r.shader for r in reqs}


def test_view_batch_at_full_size(gpu):
    pool = scenes.mesh_pool(scenes.VIEW_POOL_SPEC, seed=1)
    tex = scenes.pool_textures(4, 1024, seed=17)
    rp = hserve.ResidentPool(pool, tex)
    rp.tex_data = tex
    try:
        views = scenes.view_set(pool, 64, seed=3)
        assert max(p.mesh.nfaces for p in pool) == 1_310_720
        _check_batch(rp, views, "64 views")
    finally:
        rp.release()
