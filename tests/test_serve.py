"""GPU: replayable plans and the continuous-batching server give the same bits as the same
draws made alone, and the server's memory-based admission behaves as documented.

Every comparison is bit for bit on all three planes (colour, depth, prim ids): a request
rendered inside a mixed batch runs the same per-view arithmetic as alone, so there is no
tolerance to state.  A few requests are also checked against the oracle (depth / prim ids
bit-exact, colour within 1 LSB) to tie the server to the reference directly.
"""
import numpy as np
import pytest

import golden_io
import oracle
from hsr import scenes
from hsr import serve as hserve

pytestmark = pytest.mark.gpu

SMALL_POOL = (("grid", 32), ("sphere", 4), ("sphere", 5), ("grid", 64))


@pytest.fixture(scope="module")
def rp(gpu):
    pool = scenes.mesh_pool(SMALL_POOL, seed=21)
    tex = scenes.pool_textures(2, 256, seed=5)
    r = hserve.ResidentPool(pool, tex)
    yield r
    r.release()


def small_requests(pool, n, seed, max_side=640, fixed=None):
    """Mixed requests; `fixed=(w, h, shadow)` gives them all one target size."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        m = int(rng.integers(len(pool)))
        w = int(rng.integers(96, max_side))
        h = int(rng.integers(96, max_side))
        shader = int(scenes.REQUEST_SHADERS[int(rng.integers(len(scenes.REQUEST_SHADERS)))])
        shadow = int(rng.choice([0, 256, 512]))
        if fixed:
            w, h, shadow = fixed
        eye = scenes.orbit_eye(rng, pool[m].kind)
        sd = scenes.U.shader_data(eye, w, h, enable_shadow=bool(shadow))
        out.append(scenes.Request(m, int(rng.integers(2)), shader, w, h, shadow, sd, 0.0))
    return out


def alone(rp, r):
    """The request drawn by itself through hsr_draw_batch (shadow + main pass)."""
    vb = hserve.ViewBatch(rp, [r])
    try:
        vb.draw_all()
        return vb.download(0)
    finally:
        vb.release()


def test_plan_replay_equals_draw_batch(gpu, rp):
    views = small_requests(rp.pool, 6, seed=1)
    ref = hserve.ViewBatch(rp, views)
    got = hserve.ViewBatch(rp, views)
    try:
        ref.draw_all()
        plan = got.plan()
        try:
            for _ in range(2):  # replays are identical and equal to the direct batch
                plan.launch()
                plan.wait()
                for i in range(len(views)):
                    a, b = ref.download(i), got.download(i)
                    for p in ("color", "depth", "prim"):
                        assert np.array_equal(a[p], b[p]), (i, p)
            # new camera for view 2's main pass (and its shadow pass): replay == direct draw
            rng = np.random.default_rng(99)
            v = views[2]
            sd2 = scenes.U.shader_data(scenes.orbit_eye(rng, rp.pool[v.mesh].kind), v.width, v.height,
                                       enable_shadow=bool(v.shadow))
            k0 = sum(len(ds) for ds in got.per_view[:2])
            for k in range(len(got.per_view[2])):
                plan.set_uniforms(k0 + k, sd2)
            plan.launch()
            plan.wait()
            views2 = list(views)
            views2[2] = scenes.Request(v.mesh, v.tex, v.shader, v.width, v.height, v.shadow, sd2, 0.0)
            exp = alone(rp, views2[2])
            b = got.download(2)
            for p in ("color", "depth", "prim"):
                assert np.array_equal(exp[p], b[p]), p
            assert not np.array_equal(exp["depth"], ref.download(2)["depth"])  # the camera did move
        finally:
            plan.release()
    finally:
        ref.release()
        got.release()


def test_plan_refuses_released_handle(gpu, rp):
    views = small_requests(rp.pool, 1, seed=2)
    vb = hserve.ViewBatch(rp, views)
    plan = vb.plan()
    vb.release()
    with pytest.raises(gpu.HsrError) as e:
        plan.launch()
    assert e.value.code == gpu.ERR_BAD_HANDLE
    plan.release()


def test_server_mix_equals_alone(gpu, rp):
    reqs = small_requests(rp.pool, 40, seed=3)
    res = hserve.serve_batched(rp, reqs, pool_bytes=1 << 30, max_batch=8, slots=2, ring_bytes=64 << 20,
                               keep_outputs=True)
    assert res["ok"], res["status"]
    sizes = [res["status"][i]["batch_requests"] for i in range(len(reqs))]
    assert max(sizes) > 1, "all requests arrived at once: some batch must hold several"
    for i, r in enumerate(reqs):
        exp = alone(rp, r)
        assert np.array_equal(res["outputs"][i], exp["color"]), i


def test_long_running_server_across_calls_equals_alone(gpu, rp):
    """One server and output ring serve two streams in turn (small requests first, then larger
    ones, so its scratch grows between batches while earlier batches' copies may still run on
    their slots' streams): every request still equals the same request drawn alone."""
    small = small_requests(rp.pool, 12, seed=8, max_side=200)
    large = small_requests(rp.pool, 12, seed=9, max_side=900)
    srv = gpu.Server(1 << 30, max_batch=6, slots=2)
    ring = hserve.PinnedRing(64 << 20)
    try:
        runs = [hserve.serve_batched(rp, reqs, server=srv, ring=ring, keep_outputs=True) for reqs in (small, large)]
    finally:
        srv.close()
        ring.release()
    for reqs, res in zip((small, large), runs):
        assert res["ok"], res["status"]
        for i, r in enumerate(reqs):
            assert np.array_equal(res["outputs"][i], alone(rp, r)["color"]), i


def serve_all_planes(gpu, rp, reqs, max_batch, slots):
    """Submit every request at once and return colour / depth / prim ids of each."""
    srv = gpu.Server(1 << 30, max_batch=max_batch, slots=slots)
    try:
        outs, tickets = [], []
        for r in reqs:
            o = {"color": np.empty((r.height, r.width, 4), np.uint8), "depth": np.empty((r.height, r.width), np.float32),
                 "prim": np.empty((r.height, r.width), np.uint32)}
            d, n = rp.textures[r.tex]
            tickets.append(srv.submit(rp.meshes[r.mesh], r.shader, r.sd, r.width, r.height, diffuse=d, normal=n,
                                      shadow_size=r.shadow, clear=(hserve.BLACK, hserve.FLT_MAX),
                                      shadow_clear=(hserve.BLACK, hserve.FLT_MAX), out=o))
            outs.append(o)
        for tk in tickets:
            assert srv.wait(tk)["status"] == 0
    finally:
        srv.close()
    return outs


def test_server_depth_and_prim_equal_alone(gpu, rp):
    """All three planes through the server's own output pointers."""
    reqs = small_requests(rp.pool, 12, seed=4)
    outs = serve_all_planes(gpu, rp, reqs, max_batch=6, slots=3)
    for r, o in zip(reqs, outs):
        exp = alone(rp, r)
        for p in ("color", "depth", "prim"):
            assert np.array_equal(o[p], exp[p]), p


def test_server_vs_oracle(gpu, rp):
    reqs = small_requests(rp.pool, 4, seed=5, max_side=200)
    outs = serve_all_planes(gpu, rp, reqs, max_batch=4, slots=1)
    tex = scenes.pool_textures(2, 256, seed=5)
    for r, o in zip(reqs, outs):
        exp = oracle.render_frame(scenes.view_frame(r, rp.pool, tex))["main"]
        golden_io.assert_pass(o, {"color": exp.color, "depth": exp.depth, "prim": exp.prim}, "main",
                              f"{r.width}x{r.height} {scenes.SHADER_NAMES[r.shader]} shadow {r.shadow}")


def test_server_admission_by_memory(gpu, rp):
    reqs = small_requests(rp.pool, 8, seed=6, fixed=(200, 150, 256))
    need = 3 * (((200 * 150 * 4 + 255) // 256) * 256) + 3 * (256 * 256 * 4)
    # room for one request at a time: every batch holds exactly one request, all complete
    res = hserve.serve_batched(rp, reqs, pool_bytes=need, max_batch=8, slots=2, ring_bytes=16 << 20,
                               keep_outputs=True)
    assert res["ok"]
    assert all(res["status"][i]["batch_requests"] == 1 for i in range(len(reqs)))
    for i, r in enumerate(reqs):
        assert np.array_equal(res["outputs"][i], alone(rp, r)["color"]), i


def test_server_request_larger_than_pool_fails(gpu, rp):
    r = small_requests(rp.pool, 1, seed=7)[0]
    srv = gpu.Server(4096, max_batch=4, slots=1)
    try:
        d, n = rp.textures[r.tex]
        tk = srv.submit(rp.meshes[r.mesh], r.shader, r.sd, r.width, r.height, diffuse=d, normal=n)
        st = srv.wait(tk)
        assert st["status"] == gpu.ERR_OUT_OF_MEMORY
    finally:
        srv.close()


def test_server_rejects_bad_requests(gpu, rp):
    srv = gpu.Server(1 << 26, max_batch=4, slots=1)
    try:
        r = small_requests(rp.pool, 1, seed=8)[0]
        with pytest.raises(gpu.HsrError) as e:
            srv.submit(rp.meshes[r.mesh], 42, r.sd, 64, 64)
        assert e.value.code == gpu.ERR_UNKNOWN_SHADER
        with pytest.raises(gpu.HsrError) as e:
            srv.submit(rp.meshes[r.mesh], r.shader, r.sd, 0, 64)
        assert e.value.code == gpu.ERR_INVALID_ARG
    finally:
        srv.close()
