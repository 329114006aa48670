"""Load the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import glob
import os

import numpy as np

from hsr import scenes, uniforms as U

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


ASSET_GOLDEN = os.path.join(GOLDEN, "assets")


def asset_names() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(ASSET_GOLDEN, "*.npz")))


def load_asset(name: str):
    """A fixture of one of the reference's bundled models (tests/golden/make_golden.py assets).
    Returns (meta, expected): meta holds the model name, shader, sizes, clears, the ShaderData
    record and the SHA-256 of each asset file; expected[pass] = {depth, color, prim}."""
    import json

    z = np.load(os.path.join(ASSET_GOLDEN, name + ".npz"))
    meta = {"model": str(z["model"]), "shader": int(z["shader"]), "width": int(z["width"]),
            "height": int(z["height"]), "shadow_size": tuple(int(v) for v in z["shadow_size"]),
            "clear_rgba": tuple(int(v) for v in z["clear_rgba"]), "clear_depth": float(z["clear_depth"]),
            "shadow_clear_rgba": tuple(int(v) for v in z["shadow_clear_rgba"]),
            "shadow_clear_depth": float(z["shadow_clear_depth"]),
            "sd": np.frombuffer(z["sd"].tobytes(), U.SHADER_DATA_DTYPE).reshape(()),
            "sha256": json.loads(str(z["sha256"]))}
    exp = {}
    for k in ("main", "shadow"):
        if f"{k}_depth" in z:
            exp[k] = {"depth": z[f"{k}_depth"], "color": z[f"{k}_color"], "prim": z[f"{k}_prim"]}
    return meta, exp


def asset_files_match(meta: dict, path_of) -> bool:
    """The asset files at path_of(model, suffix) are the ones the fixture was made from."""
    import hashlib

    for suffix, digest in meta["sha256"].items():
        p = path_of(meta["model"], suffix)
        if not os.path.exists(p) or hashlib.sha256(open(p, "rb").read()).hexdigest() != digest:
            return False
    return True


def names() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name: str):
    """Returns (frame, expected) where expected[pass] = {depth, color, prim}."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    mesh = scenes.Mesh(z["pos"], z["nrm"], z["uv"], z["faces"])
    sd = np.frombuffer(z["sd"].tobytes(), U.SHADER_DATA_DTYPE).reshape(())
    fr = scenes.Frame(mesh, int(z["shader"]), sd, int(z["width"]), int(z["height"]),
                      diffuse=scenes.Texture(z["diffuse"]) if "diffuse" in z else None,
                      normal=scenes.Texture(z["normal"]) if "normal" in z else None,
                      shadow_size=tuple(int(v) for v in z["shadow_size"]),
                      clear_rgba=tuple(int(v) for v in z["clear_rgba"]), clear_depth=float(z["clear_depth"]),
                      shadow_clear_rgba=tuple(int(v) for v in z["shadow_clear_rgba"]),
                      shadow_clear_depth=float(z["shadow_clear_depth"]), name=str(z["name"]))
    exp = {}
    for k in ("main", "shadow"):
        if f"{k}_depth" in z:
            exp[k] = {"depth": z[f"{k}_depth"], "color": z[f"{k}_color"], "prim": z[f"{k}_prim"]}
    return fr, exp


def compare(got: dict, exp: dict, color_tol: int = 1) -> dict:
    """Bit-exact depth and prim ids, colour RGB within `color_tol` LSB; returns a report."""
    d_bad = int((got["depth"].view(np.uint32) != exp["depth"].view(np.uint32)).sum())
    p_bad = int((got["prim"] != exp["prim"]).sum())
    dc = np.abs(got["color"][..., :3].astype(np.int32) - exp["color"][..., :3].astype(np.int32))
    a_bad = int((got["color"][..., 3] != exp["color"][..., 3]).sum())
    return {"depth_mismatch": d_bad, "prim_mismatch": p_bad, "color_max_err": int(dc.max()) if dc.size else 0,
            "color_diff_px": int((dc.max(axis=-1) > 0).sum()), "alpha_mismatch": a_bad,
            "color_ok": bool(dc.max() <= color_tol) if dc.size else True}


def assert_pass(got: dict, exp: dict, pass_name: str, label: str = "", color_tol: int = 1) -> dict:
    """Parity of one pass against the reference (or the oracle): depth, prim ids and alpha bit
    for bit; RGB within `color_tol` LSB for the main pass (BlinnShader / NormalMapShader call
    powf, which is not correctly rounded), and bit for bit for the shadow pass (ShadowShader,
    IShader.cpp:176-180, has no powf).  Prints and returns the report: max colour error and the
    count of differing pixels."""
    rep = compare(got, exp, color_tol)
    print(label, pass_name, rep)
    assert rep["depth_mismatch"] == 0, (label, pass_name, rep)
    assert rep["prim_mismatch"] == 0, (label, pass_name, rep)
    assert rep["alpha_mismatch"] == 0, (label, pass_name, rep)
    assert rep["color_ok"], (label, pass_name, rep)
    if pass_name == "shadow":
        assert rep["color_diff_px"] == 0, (label, pass_name, rep)
    return rep
