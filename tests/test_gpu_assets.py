"""GPU: the reference's own bundled models drawn through the C ABI match the reference.

african_head (2,492 triangles) and diablo3_pose (5,022 triangles) are loaded from their
files by hsr_mesh_load_obj (normals as Model::normal returns them during the n-th draw: the
shadow pass is draw 1, the main pass draw 2, model.cpp:108-111) and hsr_texture_load_tga
(24-bit run-length maps with Model::load_texture's flip), and drawn as the reference's
application draws them (main.cpp:7-8, camera.h:8-9, scene.h:53-99): 1000x600, eye (0, 0, 2),
light (2, 2, 2); NormalMap with a 1000x600 shadow map (the published configuration on
diablo3_pose), Blinn and Toon.  Expected outputs come from the reference built headless
(tests/golden/assets).  Depth, prim ids and alpha bit for bit; RGB within 1 LSB on the main
pass and bit for bit on the shadow pass.

The asset files are not in the repository: they travel to the GPU host in oracle/_ref/assets
(copied from the reference by `make -C oracle assets`); without them the test is skipped.
"""
import pytest

import golden_io
import hsr
import refjob
from hsr import scenes

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refjob.have_assets(), reason="bundled assets not present (make -C oracle assets)")]


@pytest.mark.parametrize("name", golden_io.asset_names())
def test_bundled_model_matches_reference(gpu, name):
    meta, exp = golden_io.load_asset(name)
    assert golden_io.asset_files_match(meta, refjob.asset), "asset files differ from the fixture's"
    model = meta["model"]
    obj = refjob.asset(model, ".obj")
    shadow = meta["shadow_size"][0] > 0
    keep, objs = [], []
    try:
        # the shadow pass is the model's first draw of the frame, the main pass its next
        m_main = hsr.Mesh.from_obj(obj, hsr.OBJ_CORNER_NORMALS | hsr.obj_earlier_draws(1 if shadow else 0))
        objs.append(m_main)
        td = hsr.Texture.from_tga(refjob.asset(model, "_diffuse.tga"), hsr.TGA_MODEL_FLIP)
        tn = hsr.Texture.from_tga(refjob.asset(model, "_nm_tangent.tga"), hsr.TGA_MODEL_FLIP)
        objs += [td, tn]
        main = hsr.Target(meta["width"], meta["height"])
        objs.append(main)
        descs = []
        sm = None
        if shadow:
            m_shadow = hsr.Mesh.from_obj(obj, hsr.OBJ_CORNER_NORMALS)
            sm = hsr.Target(*meta["shadow_size"])
            objs += [m_shadow, sm]
            descs.append(hsr.make_desc(m_shadow, scenes.SHADOW, meta["sd"], sm, td, tn,
                                       clear=(meta["shadow_clear_rgba"], meta["shadow_clear_depth"]), keep=keep))
        descs.append(hsr.make_desc(m_main, meta["shader"], meta["sd"], main, td, tn, shadow_map=sm,
                                   clear=(meta["clear_rgba"], meta["clear_depth"]), keep=keep))
        hsr.draw_batch(descs)
        got = {"main": main.download()}
        if shadow:
            got["shadow"] = sm.download()
    finally:
        for o in objs:
            o.release()
    for k in exp:
        golden_io.assert_pass(got[k], exp[k], k, name)
