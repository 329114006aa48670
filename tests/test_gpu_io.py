"""GPU: assets loaded from files through the C ABI (hsr_mesh_load_obj, hsr_texture_load_tga)
render like the oracle on the same data, and the headless present (hsr_target_present,
hsr_target_write_tga) gives the image window_draw_buffer (win32.cpp:348-370) would show.

The mesh has normals that are not unit length, so the reference's in-place normalisation
(Model::normal, model.cpp:108-111) changes them on every read: the main pass of a frame reads
them after the shadow pass already normalised each once.  Tolerances as in test_gpu_parity:
depth and prim ids bit for bit, RGB within 1 LSB.
"""
import dataclasses

import numpy as np
import pytest

import golden_io
import oracle
import tga_files
from hsr import scenes

pytestmark = pytest.mark.gpu


def normals_after_draws(nrm: np.ndarray, faces: np.ndarray, draws: int) -> np.ndarray:
    """The stored normals after `draws` draws of the reference (every corner read once per
    draw, faces in order, each read normalising in place)."""
    stored = nrm.astype(np.float32).copy()
    order = faces[:, :, 2].reshape(-1)
    for _ in range(draws):
        for k in order:
            n = stored[k]
            ln = np.sqrt(np.float32(n[0] * n[0] + n[1] * n[1]) + np.float32(n[2] * n[2]), dtype=np.float32)
            n *= np.float32(1.0) / ln
    return stored


def test_loaded_obj_and_tga_render_like_the_oracle(gpu, tmp_path):
    import hsr

    fr = scenes.displaced_frame(4, 320, 240, shadow=256, tex_size=128, seed=3)
    rng = np.random.default_rng(8)
    nrm = (fr.mesh.nrm * rng.uniform(0.6, 1.7, (len(fr.mesh.nrm), 1))).astype(np.float32)
    mesh = scenes.Mesh(fr.mesh.pos, nrm, fr.mesh.uv, fr.mesh.faces)
    fr = dataclasses.replace(fr, mesh=mesh)
    obj = tmp_path / "m.obj"
    scenes.write_obj(mesh, str(obj))
    dpath, npath = tmp_path / "d.tga", tmp_path / "n.tga"
    dpath.write_bytes(tga_files.encode(fr.diffuse.data, rle=True, top_left=False))  # bottom-left origin
    hsr.tga_write(str(npath), fr.normal.data, rle=True)

    # the main pass reads normals after the shadow pass has normalised each once
    m = hsr.Mesh.from_obj(str(obj), hsr.OBJ_CORNER_NORMALS | hsr.obj_earlier_draws(1))
    td, tn = hsr.Texture.from_tga(str(dpath)), hsr.Texture.from_tga(str(npath))
    main, shadow = hsr.Target(fr.width, fr.height), hsr.Target(256, 256)
    keep = []
    try:
        d_sh = hsr.make_desc(m, scenes.SHADOW, fr.sd, shadow, td, tn, clear=(fr.shadow_clear_rgba, fr.shadow_clear_depth),
                             keep=keep)
        d_main = hsr.make_desc(m, fr.shader, fr.sd, main, td, tn, shadow_map=shadow,
                               clear=(fr.clear_rgba, fr.clear_depth), keep=keep)
        hsr.draw_batch([d_sh, d_main])
        got = {"main": main.download(), "shadow": shadow.download()}
    finally:
        for o in (main, shadow, m, td, tn):
            o.release()

    sm = oracle.Buffers(256, 256, fr.shadow_clear_rgba, fr.shadow_clear_depth)
    oracle.draw(mesh, scenes.SHADOW, fr.sd, sm, fr.diffuse, fr.normal)
    after_shadow = scenes.Mesh(mesh.pos, normals_after_draws(nrm, mesh.faces, 1), mesh.uv, mesh.faces)
    mb = oracle.Buffers(fr.width, fr.height, fr.clear_rgba, fr.clear_depth)
    oracle.draw(after_shadow, fr.shader, fr.sd, mb, fr.diffuse, fr.normal, shadow_map=sm)
    exp = {"main": {"depth": mb.depth, "color": mb.color, "prim": mb.prim},
           "shadow": {"depth": sm.depth, "color": sm.color, "prim": sm.prim}}
    for k in exp:
        golden_io.assert_pass(got[k], exp[k], k, "loaded assets")
    # the normals matter: drawn with the stored normals the image differs
    assert (got["main"]["prim"] > 0).sum() > 1000


def test_present_and_tga_dump(gpu, tmp_path):
    import hsr
    from hsr import frame as hframe

    fr = scenes.sphere_frame(3, 200, 120, shader=scenes.TEXTURE, tex_size=64, seed=4)
    g = hframe.GpuFrame(fr)
    try:
        g.render()
        col = g.main.download()["color"]
        bgr = g.main.present(3)
        bgrx = g.main.present(4)
        path = tmp_path / "frame.tga"
        g.main.write_tga(str(path), rle=True)
        g.main.write_tga(str(tmp_path / "raw.tga"), rle=False)
    finally:
        g.release()
    # window_draw_buffer: row r -> row H-1-r, bytes B, G, R
    want = col[::-1, :, [2, 1, 0]]
    assert np.array_equal(bgr, want)
    assert np.array_equal(bgrx[..., :3], want) and not bgrx[..., 3].any()
    assert np.array_equal(hsr.tga_read(str(path)), want)
    assert np.array_equal(hsr.tga_read(str(tmp_path / "raw.tga")), want)
