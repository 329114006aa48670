"""CPU: the oracle reproduces the reference on its own bundled models (african_head,
diablo3_pose: Model::Model's OBJ with normals that are not unit length, 24-bit run-length
TGA maps), in the configuration the reference's application renders them — a 1000x600
frame, eye (0, 0, 2), light (2, 2, 2), NormalMap with the shadow pass (the published
configuration on diablo3_pose), Blinn and Toon.

The fixtures hold the reference's outputs only; the asset files themselves stay outside the
repository (oracle/_ref/assets, copied from the reference by `make -C oracle assets`), so
this runs where they are present.  The main pass of a shadowed frame reads every normal
after the shadow pass has normalised it once in place (Model::normal, model.cpp:108-111):
the oracle gets the stored normals in that state and normalises on read as the reference.
"""
import numpy as np
import pytest

import golden_io
import hsr
import oracle
import refjob
from hsr import scenes

pytestmark = pytest.mark.skipif(not refjob.have_assets(), reason="bundled assets not present (make -C oracle assets)")


def stored_normals_after_draws(nrm, faces, draws):
    """Model::norms_ after `draws` draws: every face corner read once per draw, in order, each
    read normalising the stored normal in place (vector.h:41-42)."""
    stored = nrm.astype(np.float32).copy()
    for _ in range(draws):
        for k in faces[:, :, 2].reshape(-1):
            n = stored[k]
            ln = np.sqrt(np.float32(n[0] * n[0] + n[1] * n[1]) + np.float32(n[2] * n[2]), dtype=np.float32)
            n *= np.float32(1.0) / ln
    return stored


@pytest.mark.parametrize("name", golden_io.asset_names())
def test_oracle_matches_reference_on_bundled_model(name):
    meta, exp = golden_io.load_asset(name)
    assert golden_io.asset_files_match(meta, refjob.asset), "asset files differ from the fixture's"
    model = meta["model"]
    pos, nrm, uv, faces = hsr.obj_read(refjob.asset(model, ".obj"))
    diffuse = scenes.Texture(hsr.tga_read(refjob.asset(model, "_diffuse.tga"), hsr.TGA_MODEL_FLIP))
    normal = scenes.Texture(hsr.tga_read(refjob.asset(model, "_nm_tangent.tga"), hsr.TGA_MODEL_FLIP))
    sm = None
    got = {}
    if meta["shadow_size"][0] > 0:
        sm = oracle.Buffers(*meta["shadow_size"], meta["shadow_clear_rgba"], meta["shadow_clear_depth"])
        oracle.draw(scenes.Mesh(pos, nrm, uv, faces), scenes.SHADOW, meta["sd"], sm, diffuse, normal)
        got["shadow"] = {"depth": sm.depth, "color": sm.color, "prim": sm.prim}
    draws_before = 1 if sm is not None else 0
    mesh = scenes.Mesh(pos, stored_normals_after_draws(nrm, faces, draws_before), uv, faces)
    mb = oracle.Buffers(meta["width"], meta["height"], meta["clear_rgba"], meta["clear_depth"])
    oracle.draw(mesh, meta["shader"], meta["sd"], mb, diffuse, normal, shadow_map=sm)
    got["main"] = {"depth": mb.depth, "color": mb.color, "prim": mb.prim}
    for k in exp:
        golden_io.assert_pass(got[k], exp[k], k, name)
    assert (exp["main"]["prim"] > 0).sum() > 10_000
