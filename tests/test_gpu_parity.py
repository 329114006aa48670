"""GPU parity: the GB300 path through the C ABI against the reference's own outputs (golden
fixtures) and against the oracle restatement at full workload sizes.

Tolerance: depth (FP32 bits), primitive id and coverage are compared bit for bit; RGB
colour within 1 LSB per channel (powf is not correctly rounded on either side); alpha bit
for bit.  Every comparison reports the colour's max error and differing-pixel count.
"""
import numpy as np
import pytest

import golden_io
import oracle
from hsr import frame as hframe
from hsr import scenes
from hsr import uniforms as U

pytestmark = pytest.mark.gpu

COLOR_TOL = 1  # LSB per RGB channel


def gpu_render(gpu, frame, batched=True):
    g = hframe.GpuFrame(frame)
    try:
        g.render(batched=batched)
        return g.download()
    finally:
        g.release()


def assert_parity(got, exp, label):
    for k, e in exp.items():
        golden_io.assert_pass(got[k], e, k, label, COLOR_TOL)


def oracle_expect(frame):
    out = oracle.render_frame(frame)
    return {k: {"depth": v.depth, "color": v.color, "prim": v.prim} for k, v in out.items()}


@pytest.mark.parametrize("name", golden_io.names())
def test_golden_fixture(gpu, name):
    frame, exp = golden_io.load(name)
    assert_parity(gpu_render(gpu, frame), exp, name)


@pytest.mark.parametrize("tile,warps", [(8, 4), (8, 8), (16, 4), (32, 4)])
def test_tile_configs_bit_identical(gpu, tile, warps):
    frame, exp = golden_io.load("plain_frame_ico4_512_blinn")
    old = gpu.get_tuning()
    try:
        gpu.set_tuning(tile=tile, warps_per_cta=warps)
        assert_parity(gpu_render(gpu, frame), exp, f"tile{tile}x{warps}")
    finally:
        gpu.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta)


def test_batched_equals_sequential(gpu):
    frame, exp = golden_io.load("displaced4_normalmap_shadow")
    a = gpu_render(gpu, frame, batched=True)
    b = gpu_render(gpu, frame, batched=False)
    for k in a:
        for p in ("depth", "color", "prim"):
            assert np.array_equal(a[k][p], b[k][p]), (k, p)
    assert_parity(a, exp, "batched")


def test_deterministic_across_runs(gpu):
    frame, _ = golden_io.load("soup_ties_12k")
    a = gpu_render(gpu, frame)
    b = gpu_render(gpu, frame)
    for p in ("depth", "color", "prim"):
        assert np.array_equal(a["main"][p], b["main"][p])


def test_plain_frame_full_size_vs_oracle(gpu):
    frame = scenes.sphere_frame(4, 512, 512, seed=1)
    assert_parity(gpu_render(gpu, frame), oracle_expect(frame), "ico4-512")


def test_displaced_frame_1080p_shadow2048_vs_oracle(gpu):
    """The 1920x1080 frame: icosphere-7 + ground plane, NormalMap + 2048^2 shadow map."""
    frame = scenes.displaced_frame()
    assert frame.mesh.nfaces == 327_680 + 2
    assert_parity(gpu_render(gpu, frame), oracle_expect(frame), "displaced7-1080p")


def test_soup_ties_vs_oracle(gpu):
    frame = scenes.soup_frame(400_000, 1280, 720, seed=17)
    got = gpu_render(gpu, frame)
    assert_parity(got, oracle_expect(frame), "soup400k")
    # 1% exact duplicates are submitted later: each must own the pixels its original covered
    assert got["main"]["prim"].max() <= frame.mesh.nfaces


def test_soup_4m_3840x2160_vs_oracle(gpu):
    """The full depth-order stress workload: 4M triangles at 3840x2160, lognormal edges
    (median 2 px), ~8x depth complexity, 1% exact duplicates submitted later."""
    frame = scenes.soup_frame()
    assert frame.mesh.nfaces == 4_000_000 and (frame.width, frame.height) == (3840, 2160)
    got = gpu_render(gpu, frame)
    assert_parity(got, oracle_expect(frame), "soup4m-2160p")
    # the equal-depth duplicates win the pixels of their originals wherever those are visible
    faces = frame.mesh.faces[:, :, 0]
    _, first = np.unique(faces, axis=0, return_index=True)
    is_dup = np.ones(len(faces), bool)
    is_dup[first] = False
    prim = got["main"]["prim"]
    owners = prim[prim > 0].astype(np.int64) - 1
    assert is_dup[owners].sum() > 0


def test_multi_draw_same_target(gpu):
    """Two graphics_draw_triangle calls into one RenderBuffer keep the sequential depth test:
    the second draw tests against the first's depth, prim ids offset by prim_base."""
    import hsr

    fa = scenes.sphere_frame(3, 160, 120, shader=scenes.BLINN, eye=(0.2, 0.1, 2.4), tex_size=64, seed=2)
    fb = scenes.displaced_frame(3, 160, 120, shadow=0, tex_size=64, shader=scenes.TEXTURE, eye=(0.5, 0.3, 2.2))
    tgt = hsr.Target(160, 120)
    ma, mb = hsr.Mesh(fa.mesh), hsr.Mesh(fb.mesh)
    ta, tb = hsr.Texture(fa.diffuse), hsr.Texture(fb.diffuse)
    keep = []
    try:
        d1 = hsr.make_desc(ma, fa.shader, fa.sd, tgt, ta, clear=(fa.clear_rgba, fa.clear_depth), keep=keep)
        d2 = hsr.make_desc(mb, fb.shader, fb.sd, tgt, tb, prim_base=1_000_000, keep=keep)
        hsr.draw_batch([d1, d2])
        got = tgt.download()
        # the same sequence through two separate calls
        hsr.draw(d1)
        hsr.draw(d2)
        got2 = tgt.download()
    finally:
        for o in (tgt, ma, mb, ta, tb):
            o.release()
    rb = oracle.Buffers(160, 120, fa.clear_rgba, fa.clear_depth)
    oracle.draw(fa.mesh, fa.shader, fa.sd, rb, fa.diffuse)
    oracle.draw(fb.mesh, fb.shader, fb.sd, rb, fb.diffuse, prim_base=1_000_000)
    exp = {"main": {"depth": rb.depth, "color": rb.color, "prim": rb.prim}}
    assert_parity({"main": got}, exp, "multi-draw batch")
    assert_parity({"main": got2}, exp, "multi-draw calls")


def test_a_second_clear_of_a_target_follows_the_earlier_draws(gpu):
    """[A clear, B clear, C] into one target, as one batch and as three calls, equals the
    reference's sequence: B's clear erases A, then B and C draw (C tests against B's depth).
    The batch runs as two launch sequences, split before B; a plan (one launch sequence)
    refuses it."""
    import hsr

    fa = scenes.sphere_frame(3, 160, 120, shader=scenes.BLINN, eye=(0.2, 0.1, 2.4), tex_size=64, seed=2)
    fb = scenes.displaced_frame(3, 160, 120, shadow=0, tex_size=64, shader=scenes.TEXTURE, eye=(0.5, 0.3, 2.2))
    fc = scenes.sphere_frame(3, 160, 120, shader=scenes.TOON, eye=(-0.4, 0.2, 2.0), tex_size=64, seed=7)
    b_clear = ((10, 20, 30, 40), 100.0)
    tgt = hsr.Target(160, 120)
    ma, mb, mc = hsr.Mesh(fa.mesh), hsr.Mesh(fb.mesh), hsr.Mesh(fc.mesh)
    ta, tb, tc = hsr.Texture(fa.diffuse), hsr.Texture(fb.diffuse), hsr.Texture(fc.diffuse)
    keep = []
    try:
        d1 = hsr.make_desc(ma, fa.shader, fa.sd, tgt, ta, clear=(fa.clear_rgba, fa.clear_depth), keep=keep)
        d2 = hsr.make_desc(mb, fb.shader, fb.sd, tgt, tb, clear=b_clear, prim_base=1_000_000, keep=keep)
        d3 = hsr.make_desc(mc, fc.shader, fc.sd, tgt, tc, prim_base=2_000_000, keep=keep)
        hsr.draw_batch([d1, d2, d3])
        got = tgt.download()
        for d in (d1, d2, d3):
            hsr.draw(d)
        got2 = tgt.download()
        with pytest.raises(gpu.HsrError) as e:
            hsr.Plan([d1, d2, d3])
        assert e.value.code == gpu.ERR_INVALID_ARG
    finally:
        for o in (tgt, ma, mb, mc, ta, tb, tc):
            o.release()
    rb = oracle.Buffers(160, 120, *b_clear)
    oracle.draw(fb.mesh, fb.shader, fb.sd, rb, fb.diffuse, prim_base=1_000_000)
    oracle.draw(fc.mesh, fc.shader, fc.sd, rb, fc.diffuse, prim_base=2_000_000)
    exp = {"main": {"depth": rb.depth, "color": rb.color, "prim": rb.prim}}
    assert_parity({"main": got}, exp, "re-clear batch")
    assert_parity({"main": got2}, exp, "re-clear calls")


def test_draw_without_clear_keeps_untouched_pixels(gpu):
    import hsr

    frame = scenes.sphere_frame(3, 64, 48, shader=scenes.TEXTURE, tex_size=16, seed=5)
    rng = np.random.default_rng(0)
    color = rng.integers(0, 256, (48, 64, 4), dtype=np.uint8)
    depth = rng.uniform(0.9, 1.1, (48, 64)).astype(np.float32)
    prim = rng.integers(0, 1000, (48, 64), dtype=np.uint32)
    tgt = hsr.Target(64, 48)
    m, t = hsr.Mesh(frame.mesh), hsr.Texture(frame.diffuse)
    keep = []
    try:
        tgt.upload(color, depth, prim)
        hsr.draw(hsr.make_desc(m, frame.shader, frame.sd, tgt, t, keep=keep))
        got = tgt.download()
    finally:
        for o in (tgt, m, t):
            o.release()
    rb = oracle.Buffers(64, 48)
    rb.color[:] = color
    rb.depth[:] = depth
    rb.prim[:] = prim
    oracle.draw(frame.mesh, frame.shader, frame.sd, rb, frame.diffuse)
    assert_parity({"main": got}, {"main": {"depth": rb.depth, "color": rb.color, "prim": rb.prim}}, "no-clear")


def test_scratch_overflow_retries_and_stays_exact(gpu):
    frame, exp = golden_io.load("soup_ties_12k")
    old = gpu.get_tuning()
    import hsr
    import hsr as _h

    try:
        # a fresh runtime forgets capacity hints learnt from earlier tests
        _h.shutdown()
        _h.init(0)
        gpu.set_tuning(bin_factor=0.5)
        got = gpu_render(gpu, frame)
        st = hsr.stats()
    finally:
        gpu.set_tuning(bin_factor=old.bin_factor)
    assert_parity(got, exp, "overflow-retry")
    assert st["bin_pairs"] > 0


def test_errors_are_status_codes(gpu):
    import ctypes

    import hsr

    frame = scenes.sphere_frame(2, 32, 32, tex_size=8)
    m, tgt = hsr.Mesh(frame.mesh), hsr.Target(32, 32)
    keep = []
    try:
        d = hsr.make_desc(m, 99, frame.sd, tgt, keep=keep)
        with pytest.raises(hsr.HsrError) as e:
            hsr.draw(d)
        assert e.value.code == hsr.ERR_UNKNOWN_SHADER
        d = hsr.make_desc(m, scenes.BLINN, frame.sd, tgt, keep=keep)
        d.target = 123456789
        with pytest.raises(hsr.HsrError) as e:
            hsr.draw(d)
        assert e.value.code == hsr.ERR_BAD_HANDLE
        bad = frame.mesh.faces.copy()
        bad[0, 0, 0] = len(frame.mesh.pos)
        with pytest.raises(hsr.HsrError) as e:
            hsr.Mesh(scenes.Mesh(frame.mesh.pos, frame.mesh.nrm, frame.mesh.uv, bad))
        assert e.value.code == hsr.ERR_INVALID_ARG
        h = ctypes.c_uint64()
        assert hsr.lib().hsr_target_create(0, 10, ctypes.byref(h)) == hsr.ERR_INVALID_ARG
    finally:
        m.release()
        tgt.release()


def test_empty_mesh_only_clears(gpu):
    import hsr

    mesh = scenes.Mesh(np.zeros((1, 3), np.float32), np.array([[0, 0, 1]], np.float32),
                       np.zeros((1, 2), np.float32), np.zeros((0, 3, 3), np.int32))
    frame = scenes.sphere_frame(2, 40, 30, tex_size=8)
    m, tgt = hsr.Mesh(mesh), hsr.Target(40, 30)
    keep = []
    try:
        hsr.draw(hsr.make_desc(m, scenes.BLINN, frame.sd, tgt, clear=((1, 2, 3, 4), 0.5), keep=keep))
        got = tgt.download()
    finally:
        m.release()
        tgt.release()
    assert (got["color"] == np.array([1, 2, 3, 4], np.uint8)).all()
    assert (got["depth"] == np.float32(0.5)).all() and (got["prim"] == 0).all()


def _light_far_frame():
    """A shadowed frame whose shadow pass has no triangle: the light sits 40 units out, beyond
    the far plane of its orthographic volume (depth 0..5), while the camera sees the mesh."""
    f = scenes.sphere_frame(3, 96, 72, shader=scenes.BLINN, tex_size=32, seed=3, shadow=64)
    f.sd = U.shader_data((0.0, 0.0, 3.0), 96, 72, light=(0.0, 0.0, 40.0), enable_shadow=True)
    f.name = "light_far"
    return f


def _looking_away_frame():
    """A shadowed frame whose main pass has no triangle (every face is behind the camera)
    while its shadow pass has many: all main pixels come from the clear of empty tiles."""
    f = scenes.sphere_frame(3, 80, 64, shader=scenes.NORMALMAP, tex_size=32, seed=4, shadow=64, nm_size=16)
    f.sd = U.shader_data((0.0, 0.0, 3.0), 80, 64, target=(0.0, 0.0, 6.0), enable_shadow=True)
    f.name = "looking_away"
    return f


@pytest.mark.parametrize("make", [_light_far_frame, _looking_away_frame])
def test_views_without_triangles_vs_oracle(gpu, make):
    """A view with no triangle has no tile in the raster's list: its pixels come from the
    clear that runs beside the binning, and a view waiting on it (the main pass on its shadow
    map) waits for nothing."""
    fr = make()
    exp = oracle_expect(fr)
    assert_parity(gpu_render(gpu, fr, batched=True), exp, fr.name + " batched")
    assert_parity(gpu_render(gpu, fr, batched=False), exp, fr.name + " per pass")


def test_batch_mixing_empty_and_full_views_vs_oracle(gpu):
    """One launch sequence over frames whose shadow or main pass is empty and a normal frame,
    each with its own targets: the non-empty tile list spans views with and without
    triangles, and each main pass waits on its own shadow map only."""
    import hsr

    frames = [_light_far_frame(), scenes.sphere_frame(3, 72, 56, shader=scenes.TOON, tex_size=16, seed=6, shadow=32),
              _looking_away_frame()]
    gfs = [hframe.GpuFrame(f) for f in frames]
    try:
        hsr.draw_batch([d for g in gfs for d in g.descs])
        got = [g.download() for g in gfs]
    finally:
        for g in gfs:
            g.release()
    for f, g in zip(frames, got):
        assert_parity(g, oracle_expect(f), f.name + " in a mixed batch")


def test_autotune_picks_a_valid_config_and_stays_exact(gpu):
    import hsr

    frame, exp = golden_io.load("displaced4_normalmap_shadow")
    old = gpu.get_tuning()
    g = hframe.GpuFrame(frame)
    try:
        best = hsr.autotune(g.descs, reps=2)
        assert best["tile"] in (8, 16, 32) and best["warps_per_cta"] in (4, 8) and 1 <= best["ctas_per_sm"] <= 8
        assert 0.5 <= best["bin_factor"] <= 64.0
        g.render()
        got = g.download()
    finally:
        g.release()
        gpu.set_tuning(tile=old.tile, warps_per_cta=old.warps_per_cta, ctas_per_sm=old.ctas_per_sm,
                       bin_factor=old.bin_factor)
    assert_parity(got, exp, f"autotuned {best}")
