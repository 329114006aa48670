"""GPU: the failure paths report a status and leave the device usable.

No GPU is faulted, trapped or hung here.  The failures are made on the host:
  - hsr_set_fault_injection lowers the poll limit of the bounded device waits and makes one
    of them wait for something nothing provides (a shadow map tile that never finishes; a scan
    prefix that is never published).  The wait runs out, the kernel returns, the call reports
    HSR_ERR_TIMEOUT, and the next draw on the same context is exact again;
  - hsr_server_inject_alloc_failures makes the server's target allocations fail as if the
    memory pool were exhausted: the requests are deferred and complete once allocations
    succeed, or fail with HSR_ERR_OUT_OF_MEMORY when they never can.
Reference: the reference reports no errors at all (graphics.cpp asserts only); these are the
status codes the C ABI adds.
"""
import time

import numpy as np
import pytest

import golden_io
import oracle
from hsr import frame as hframe
from hsr import scenes
from hsr import serve as hserve

pytestmark = pytest.mark.gpu


def _expect(frame):
    out = oracle.render_frame(frame)
    return {k: {"depth": v.depth, "color": v.color, "prim": v.prim} for k, v in out.items()}


@pytest.fixture
def faults(gpu):
    yield gpu
    gpu.set_fault_injection(0, 0)


def test_dependency_wait_runs_out_and_the_next_draw_is_exact(faults):
    gpu = faults
    fr = scenes.displaced_frame(4, 320, 240, shadow=256, tex_size=64, seed=3)
    g = hframe.GpuFrame(fr)
    try:
        gpu.set_fault_injection(gpu.FAULT_DEPENDENCY_STALL, 4000)
        t0 = time.perf_counter()
        with pytest.raises(gpu.HsrError) as e:
            g.render(batched=True)  # the main pass waits on the shadow pass inside one launch sequence
        waited = time.perf_counter() - t0
        assert e.value.code == gpu.ERR_TIMEOUT
        assert waited < 10.0, waited  # one limit, not one per tile
        gpu.set_fault_injection(0, 0)
        g.render(batched=True)
        got = g.download()
    finally:
        g.release()
    exp = _expect(fr)
    for k in exp:
        golden_io.assert_pass(got[k], exp[k], k, "after a dependency timeout")


def test_scan_lookback_runs_out_and_no_target_is_written(faults):
    gpu = faults
    old = gpu.get_tuning()
    # 1280x720 in 8x8 tiles: 14,400 tiles, eight scan blocks, so the look-back has predecessors
    fr = scenes.sphere_frame(4, 1280, 720, shader=scenes.BLINN, tex_size=64, seed=2)
    g = hframe.GpuFrame(fr)
    try:
        gpu.set_tuning(tile=8, warps_per_cta=4)
        g.main.clear((7, 7, 7, 7), 0.5)
        before = g.main.download()
        gpu.set_fault_injection(gpu.FAULT_SCAN_STALL, 4000)
        with pytest.raises(gpu.HsrError) as e:
            g.render()
        assert e.value.code == gpu.ERR_TIMEOUT
        after = g.main.download()
        for p in ("color", "depth", "prim"):
            assert np.array_equal(before[p], after[p]), p  # the stalled sequence drew nothing
        gpu.set_fault_injection(0, 0)
        g.render()
        got = g.download()
    finally:
        g.release()
        gpu.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta)
    golden_io.assert_pass(got["main"], _expect(fr)["main"], "main", "after a scan timeout")


def test_fault_injection_rejects_unknown_bits(gpu):
    with pytest.raises(gpu.HsrError) as e:
        gpu.set_fault_injection(1 << 7, 0)
    assert e.value.code == gpu.ERR_INVALID_ARG
    with pytest.raises(gpu.HsrError) as e:
        gpu.set_fault_injection(0, -1)
    assert e.value.code == gpu.ERR_INVALID_ARG


@pytest.fixture(scope="module")
def rp(gpu):
    pool = scenes.mesh_pool((("grid", 32), ("sphere", 4), ("sphere", 5)), seed=31)
    tex = scenes.pool_textures(2, 128, seed=7)
    r = hserve.ResidentPool(pool, tex)
    yield r
    r.release()


def _requests(pool, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        m = int(rng.integers(len(pool)))
        w, h = int(rng.integers(96, 320)), int(rng.integers(96, 320))
        shader = int(scenes.REQUEST_SHADERS[int(rng.integers(len(scenes.REQUEST_SHADERS)))])
        shadow = int(rng.choice([0, 256]))
        sd = scenes.U.shader_data(scenes.orbit_eye(rng, pool[m].kind), w, h, enable_shadow=bool(shadow))
        out.append(scenes.Request(m, int(rng.integers(2)), shader, w, h, shadow, sd, 0.0))
    return out


def _alone(rp, r):
    vb = hserve.ViewBatch(rp, [r])
    try:
        vb.draw_all()
        return vb.download(0)
    finally:
        vb.release()


def _serve(gpu, rp, reqs, inject):
    srv = gpu.Server(1 << 30, 8, 2)
    outs = [np.zeros((r.height, r.width, 4), np.uint8) for r in reqs]
    try:
        srv.inject_alloc_failures(inject)
        tks = [srv.submit(rp.meshes[r.mesh], r.shader, r.sd, r.width, r.height, diffuse=rp.textures[r.tex][0],
                          normal=rp.textures[r.tex][1], shadow_size=r.shadow, out={"color": o})
               for r, o in zip(reqs, outs)]
        sts = [srv.wait(t, 60000) for t in tks]
    finally:
        srv.close()
    return sts, outs


def test_server_defers_requests_whose_targets_cannot_be_allocated(gpu, rp):
    reqs = _requests(rp.pool, 6, seed=1)
    sts, outs = _serve(gpu, rp, reqs, inject=3)
    assert all(st["status"] == gpu.OK for st in sts), sts
    assert sts[0]["deferred"] >= 1, sts  # the first admission attempts failed and were retried
    for r, o in zip(reqs, outs):
        assert np.array_equal(o, _alone(rp, r)["color"])


def test_server_fails_a_request_that_never_gets_memory(gpu, rp):
    """With no batch in flight, the head request gets 8 attempts; then it alone fails with
    HSR_ERR_OUT_OF_MEMORY and the requests behind it are served."""
    reqs = _requests(rp.pool, 4, seed=2)
    sts, outs = _serve(gpu, rp, reqs, inject=8)
    assert sts[0]["status"] == gpu.ERR_OUT_OF_MEMORY, sts
    assert all(st["status"] == gpu.OK for st in sts[1:]), sts
    for r, o in zip(reqs[1:], outs[1:]):
        assert np.array_equal(o, _alone(rp, r)["color"])
