"""Generate the golden fixtures of the draw path from the reference itself.

Run where the reference sources are present (it builds oracle/_ref/ref_harness from them):

    python tests/golden/make_golden.py

Each fixture stores its inputs (mesh arrays, textures, the ShaderData record as bytes,
sizes, clear values) and the reference's outputs per pass: FP32 depth, RGBA8 colour and
the primitive-id plane (face + 1, 0 = untouched) from a PrimIdShader run on the same
geometry.  Inputs are stored rather than regenerated so that the fixtures do not depend
on the host's libm (spherical uvs use atan2/asin).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "hana-softwarerenderer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from hsr import scenes, uniforms as U  # noqa: E402
import refjob  # noqa: E402

F32 = np.float32


def integer_grid_frame(n: int = 64, cells: int = 8) -> scenes.Frame:
    """Coplanar quads whose vertices land exactly on pixel sample points: inclusive edges and
    equal-depth ties on every shared edge (the later triangle must win)."""
    step = n // cells
    xs = np.arange(cells + 1) * step
    X, Y = np.meshgrid(xs, xs)
    ndc = lambda p: (p.astype(np.float64) * 2.0 / n - 1.0)  # noqa: E731  exact for powers of two
    pos = np.stack([ndc(X.ravel()), ndc(Y.ravel()), np.full(X.size, 0.25)], 1).astype(np.float32)
    idx = np.arange(X.size).reshape(cells + 1, cells + 1)
    a, b = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
    c, d = idx[1:, 1:].ravel(), idx[1:, :-1].ravel()
    tri = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)])
    faces = np.zeros((len(tri), 3, 3), np.int32)
    faces[:, :, 0] = tri
    mesh = scenes.Mesh(pos, np.array([[0, 0, 1]], np.float32), np.zeros((1, 2), np.float32), faces)
    sd = U.shader_data((0, 0, 1), n, n, identity_mvp=True)
    return scenes.Frame(mesh, scenes.FLAT, sd, n, n, name="integer_grid")


def degenerate_frame() -> scenes.Frame:
    """Slivers with |u.z| <= 0.01, zero-area and back-facing triangles among normal ones."""
    rng = np.random.default_rng(5)
    W = H = 48
    cross2 = lambda a, b: a[0] * b[1] - a[1] * b[0]  # noqa: E731
    tris = []
    for _ in range(60):
        c = rng.uniform(-0.9, 0.9, 2)
        kind = rng.integers(0, 4)
        if kind == 0:   # normal CCW
            p = c + rng.uniform(-0.2, 0.2, (3, 2))
            if cross2(p[1] - p[0], p[2] - p[0]) < 0:
                p = p[[0, 2, 1]]
        elif kind == 1:  # sliver: tiny area
            d = rng.uniform(-0.2, 0.2, 2)
            p = np.stack([c, c + d, c + d * 0.5 + np.array([1e-4, -1e-4])])
        elif kind == 2:  # zero area
            d = rng.uniform(-0.2, 0.2, 2)
            p = np.stack([c, c + d, c + 2 * d])
        else:            # back-facing
            p = c + rng.uniform(-0.2, 0.2, (3, 2))
            if cross2(p[1] - p[0], p[2] - p[0]) > 0:
                p = p[[0, 2, 1]]
        z = rng.uniform(0, 0.9)
        tris.append(np.concatenate([p, np.full((3, 1), z)], 1))
    pos = np.concatenate(tris).astype(np.float32)
    faces = np.zeros((len(tris), 3, 3), np.int32)
    faces[:, :, 0] = np.arange(len(pos)).reshape(-1, 3)
    mesh = scenes.Mesh(pos, np.array([[0, 0, 1]], np.float32), np.zeros((1, 2), np.float32), faces)
    sd = U.shader_data((0, 0, 1), W, H, identity_mvp=True)
    return scenes.Frame(mesh, scenes.FLAT, sd, W, H, name="degenerate")


def fixtures():
    out = []
    for sh in range(7):
        fr = scenes.sphere_frame(3, 96, 72, shader=sh, tex_size=32, nm_size=32, seed=3 + sh)
        fr.name = f"sphere3_{scenes.SHADER_NAMES[sh]}"
        out.append(fr)
    fr = scenes.sphere_frame(4, 512, 512)
    fr.name = "plain_frame_ico4_512_blinn"
    out.append(fr)
    for sh in (scenes.BLINN, scenes.NORMALMAP, scenes.TEXTURE_WITH_LIGHT):
        fr = scenes.sphere_frame(3, 160, 120, shader=sh, eye=(0.3, 0.2, 1.25), tex_size=64, nm_size=64, seed=21)
        fr.name = f"clip_close_{scenes.SHADER_NAMES[sh]}"
        out.append(fr)
    fr = scenes.displaced_frame(4, 240, 135, shadow=256, tex_size=128)
    fr.name = "displaced4_normalmap_shadow"
    out.append(fr)
    fr = scenes.displaced_frame(4, 200, 120, shadow=128, tex_size=64, shader=scenes.BLINN, eye=(0.6, 1.4, 2.6))
    fr.name = "displaced4_blinn_shadow"
    out.append(fr)
    fr = scenes.displaced_frame(3, 160, 90, shadow=0, tex_size=64, shader=scenes.TOON)
    fr.name = "displaced3_toon_plane"
    out.append(fr)
    fr = scenes.soup_frame(12000, 256, 160, seed=4)
    fr.name = "soup_ties_12k"
    out.append(fr)
    # texture formats: 1-byte diffuse (TGAColor(p,1) -> B only), 3-byte diffuse
    fr = scenes.sphere_frame(3, 96, 96, shader=scenes.TEXTURE, tex_size=48, seed=9)
    fr.diffuse = scenes.noise_texture(48, 48, 1, 9)
    fr.name = "texture_bpp1"
    out.append(fr)
    fr = scenes.sphere_frame(3, 96, 96, shader=scenes.TEXTURE_WITH_LIGHT, tex_size=48, seed=10)
    fr.diffuse = scenes.noise_texture(48, 48, 3, 10)
    fr.name = "texture_bpp3"
    out.append(fr)
    # RenderBuffer constructor state: colour (0,0,0,255), depth 1.0 (renderbuffer.cpp:3-18)
    fr = scenes.sphere_frame(3, 128, 128, shader=scenes.GROUND, seed=12, eye=(0.5, 0.5, 2.2), tex_size=32)
    fr.clear_rgba = (0, 0, 0, 255)
    fr.clear_depth = 1.0
    fr.name = "ctor_clear_depth1"
    out.append(fr)
    # a clear depth that rejects part of the surface
    fr = scenes.sphere_frame(3, 96, 96, shader=scenes.BLINN, seed=13, eye=(0, 0, 2.0), tex_size=64)
    fr.clear_depth = 0.9997
    fr.clear_rgba = (10, 20, 30, 40)
    fr.name = "partial_depth_reject"
    out.append(fr)
    out.append(integer_grid_frame())
    out.append(degenerate_frame())
    return out


# The reference's bundled models in the configuration its application renders them
# (main.cpp:7-8: a 1000x600 frame; camera.h:8-9: eye (0, 0, 2) looking at the origin; the light
# at (2, 2, 2), scene.cpp:7; Material White / White / gloss 50 / bump 1, scene.cpp:81-84;
# the shadow map a RenderBuffer of the frame's size, scene.h:78), with the shaders of its
# shader list (scene.cpp:87-97).  The first is the published configuration: diablo3_pose,
# NormalMapShader with the shadow pass.
ASSET_SCENES = (("diablo3_pose", scenes.NORMALMAP, True), ("african_head", scenes.NORMALMAP, True),
                ("african_head", scenes.BLINN, False), ("diablo3_pose", scenes.TOON, False))
ASSET_W, ASSET_H = 1000, 600


def asset_frame(model: str, shader: int, shadow: bool) -> scenes.Frame:
    """The frame of one bundled model: mesh arrays as Model::Model parses the OBJ (for the
    prim-id run), maps as TGAImage reads them with Model::load_texture's flip."""
    import hsr

    pos, nrm, uv, faces = hsr.obj_read(refjob.asset(model, ".obj"))
    mesh = scenes.Mesh(pos, nrm, uv, faces)
    diffuse = scenes.Texture(refjob.ref_tga_read(refjob.asset(model, "_diffuse.tga"), True))
    normal = scenes.Texture(refjob.ref_tga_read(refjob.asset(model, "_nm_tangent.tga"), True))
    sd = U.shader_data((0.0, 0.0, 2.0), ASSET_W, ASSET_H, enable_shadow=shadow)
    return scenes.Frame(mesh, shader, sd, ASSET_W, ASSET_H, diffuse=diffuse, normal=normal,
                        shadow_size=(ASSET_W, ASSET_H) if shadow else (0, 0),
                        name=f"asset_{model}_{scenes.SHADER_NAMES[shader]}{'_shadow' if shadow else ''}")


def asset_sha256(model: str) -> dict:
    import hashlib

    return {s: hashlib.sha256(open(refjob.asset(model, s), "rb").read()).hexdigest()
            for s in (".obj", "_diffuse.tga", "_nm_tangent.tga")}


def save_asset(model: str, shader: int, shadow: bool, path: str) -> dict:
    """Outputs only (the assets are not copied into the repository): the reference's draw of
    the model's own OBJ, the prim ids from the PrimIdShader run on the same positions, the
    ShaderData bits, and the SHA-256 of each asset file the frame reads."""
    import json

    frame = asset_frame(model, shader, shadow)
    ref = refjob.run(frame, obj_path=refjob.asset(model, ".obj"))
    ids = refjob.run_prim_ids(frame)
    arrays = {
        "name": np.array(frame.name), "model": np.array(model), "shader": np.int32(shader),
        "width": np.int32(frame.width), "height": np.int32(frame.height),
        "shadow_size": np.array(frame.shadow_size, np.int32),
        "clear_rgba": np.array(frame.clear_rgba, np.uint8), "clear_depth": np.float32(frame.clear_depth),
        "shadow_clear_rgba": np.array(frame.shadow_clear_rgba, np.uint8),
        "shadow_clear_depth": np.float32(frame.shadow_clear_depth),
        "sd": np.frombuffer(np.ascontiguousarray(frame.sd).tobytes(), np.uint8),
        "sha256": np.array(json.dumps(asset_sha256(model))),
    }
    info = {}
    for k, v in ref.items():
        if not (ids[k]["depth"].view(np.uint32) == v["depth"].view(np.uint32)).all():
            raise RuntimeError(f"{frame.name}/{k}: prim-id run changed coverage or depth")
        arrays[f"{k}_depth"] = v["depth"]
        arrays[f"{k}_color"] = v["color"]
        arrays[f"{k}_prim"] = ids[k]["prim"]
        info[k] = int((ids[k]["prim"] > 0).sum())
    np.savez_compressed(path, **arrays)
    return info


def save(frame, path: str) -> dict:
    ref = refjob.run(frame)
    ids = refjob.run_prim_ids(frame)
    arrays = {
        "name": np.array(frame.name), "shader": np.int32(frame.shader),
        "width": np.int32(frame.width), "height": np.int32(frame.height),
        "shadow_size": np.array(frame.shadow_size, np.int32),
        "clear_rgba": np.array(frame.clear_rgba, np.uint8), "clear_depth": np.float32(frame.clear_depth),
        "shadow_clear_rgba": np.array(frame.shadow_clear_rgba, np.uint8),
        "shadow_clear_depth": np.float32(frame.shadow_clear_depth),
        "sd": np.frombuffer(np.ascontiguousarray(frame.sd).tobytes(), np.uint8),
        "pos": frame.mesh.pos, "nrm": frame.mesh.nrm, "uv": frame.mesh.uv, "faces": frame.mesh.faces,
    }
    if frame.diffuse is not None:
        arrays["diffuse"] = frame.diffuse.data
    if frame.normal is not None:
        arrays["normal"] = frame.normal.data
    info = {}
    for k, v in ref.items():
        same = (ids[k]["depth"].view(np.uint32) == v["depth"].view(np.uint32)).all()
        if not same:
            raise RuntimeError(f"{frame.name}/{k}: prim-id run changed coverage or depth")
        arrays[f"{k}_depth"] = v["depth"]
        arrays[f"{k}_color"] = v["color"]
        arrays[f"{k}_prim"] = ids[k]["prim"]
        info[k] = int((ids[k]["prim"] > 0).sum())
    np.savez_compressed(path, **arrays)
    return info


def matrices(path: str) -> None:
    """Matrix builders of the reference (maths.cpp) for a few cameras and aspects."""
    rows = []
    params = [((0, 0, 3), 512, 512), ((0, 0.8, 3.2), 1920, 1080), ((1.3, -0.4, 2.1), 1280, 720),
              ((-2.0, 1.5, -1.0), 256, 256), ((0.0, 3.0, 0.01), 640, 480)]
    for eye, w, h in params:
        asp = F32(F32(w) / F32(h))
        r = refjob.ref_matrices(eye, (0, 0, 0), (0, 1, 0), U.FOVY, asp, U.NEAR, U.FAR, U.LIGHT_POS, (asp, 1, 0, 5))
        rows.append(np.concatenate([np.array(eye, np.float32), np.array([w, h], np.float32), r["view"], r["proj"],
                                    r["camera_vp"], r["light_vp"], r["model_I"], r["light_dir"]]))
    np.save(path, np.stack(rows).astype(np.float32))


def camera_cases(n: int = 200, seed: int = 31) -> np.ndarray:
    """Inputs of Camera::update_transform: position, target, orbit, pan, dolly.  Random orbits
    around a target near the origin, plus the edge cases of the reference's formulas: the eye
    straight above / below the target (azimuth of (0, 0), polar angle clamped), orbits past the
    poles, no motion, and large dolly steps either way."""
    rng = np.random.default_rng(seed)
    pos = rng.normal(0, 1, (n, 3))
    pos *= rng.uniform(0.3, 6.0, (n, 1)) / np.linalg.norm(pos, axis=1, keepdims=True)
    target = rng.uniform(-1, 1, (n, 3)) * (rng.random((n, 1)) < 0.7)
    rows = np.concatenate([pos + target, target, rng.uniform(-0.6, 0.6, (n, 2)), rng.uniform(-0.3, 0.3, (n, 2)),
                           rng.uniform(-12, 12, (n, 1)).round(0) * (rng.random((n, 1)) < 0.8)], axis=1)
    special = [
        [0, 2, 0, 0, 0, 0, 0.1, 0.05, 0.02, -0.01, 1],    # straight above the target
        [0, -3, 0, 0, 0, 0, -0.2, -0.3, 0, 0, -2],        # straight below
        [0, 0, 2, 0, 0, 0, 0, 0.9, 0, 0, 0],              # orbit past the north pole (clamped)
        [0, 0, 2, 0, 0, 0, 0, -0.9, 0, 0, 0],             # past the south pole
        [1.5, 0.5, -2, 0.25, -0.5, 0.125, 0, 0, 0, 0, 0],  # no motion
        [0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 40],               # dolly far in
        [0, 0, 2, 0, 0, 0, 0, 0, 0, 0, -40],              # dolly far out
        [0.5, 1, 2, 0, 0, 0, 0.25, 0.1, 0.2, -0.15, 3.5],  # fractional dolly
    ]
    return np.concatenate([rows, np.array(special, np.float64)]).astype(np.float32)


def camera(path: str) -> None:
    """Camera::update_transform of the reference (camera.cpp:63-70): inputs and outputs."""
    cases = camera_cases()
    np.save(path, np.concatenate([cases, refjob.ref_camera(cases)], axis=1).astype(np.float32))


def main() -> None:
    """`make_golden.py` writes every fixture; `make_golden.py frames|matrices|camera|assets ...`
    only the named groups (assets: outputs of the bundled models, under tests/golden/assets)."""
    if not refjob.build():
        raise SystemExit("reference sources not found; fixtures can only be generated where they exist")
    want = set(sys.argv[1:]) or {"frames", "matrices", "camera", "assets"}
    total = 0
    if "assets" in want:
        if not refjob.have_assets():
            raise SystemExit("bundled assets not copied to oracle/_ref/assets (make -C oracle assets)")
        os.makedirs(os.path.join(HERE, "assets"), exist_ok=True)
        for model, shader, shadow in ASSET_SCENES:
            p = os.path.join(HERE, "assets", f"{model}_{scenes.SHADER_NAMES[shader]}{'_shadow' if shadow else ''}.npz")
            info = save_asset(model, shader, shadow, p)
            sz = os.path.getsize(p)
            total += sz
            print(f"{os.path.basename(p):40s} covered={info} {sz/1024:.0f} KiB")
    if "frames" in want:
        for fr in fixtures():
            p = os.path.join(HERE, fr.name + ".npz")
            info = save(fr, p)
            sz = os.path.getsize(p)
            total += sz
            print(f"{fr.name:32s} faces={fr.mesh.nfaces:7d} covered={info} {sz/1024:.0f} KiB")
    if "matrices" in want:
        matrices(os.path.join(HERE, "matrices.npy"))
    if "camera" in want:
        camera(os.path.join(HERE, "camera_update.npy"))
    print(f"total {total/1024:.0f} KiB")


if __name__ == "__main__":
    main()
