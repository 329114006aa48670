"""Driver for oracle/_ref/ref_harness — TEST INFRASTRUCTURE ONLY.

Writes a job file (format documented in oracle/ref_harness.cpp), runs the reference's own
draw path compiled headless, and reads the buffers back.  Used to generate the golden
fixtures under tests/golden/ and to pin the C restatement (oracle/hsr_oracle.c) against
the reference where the reference sources are available.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "ref_harness")
SHIM_HOST_HARNESS = os.path.join(HERE, "_ref", "ref_harness_shim_host")
# The reference's source tree (read only): HSR_REFERENCE_DIR, else where it is unpacked on the
# build host.  Hosts without it (the GPU hosts) use what `build` left in oracle/_ref.
REF_DIR = os.environ.get("HSR_REFERENCE_DIR", "/root/reference/Hana-SoftwareRenderer")
# Copies of the reference's bundled models and maps (make assets), kept out of the repository
ASSETS = os.path.join(HERE, "_ref", "assets")


def available() -> bool:
    return os.path.exists(HARNESS)


def have_reference() -> bool:
    return os.path.isdir(REF_DIR)


def asset(model: str, suffix: str) -> str:
    """Path of a bundled asset file in oracle/_ref/assets (e.g. asset("diablo3_pose", ".obj"))."""
    return os.path.join(ASSETS, model, model + suffix)


def have_assets() -> bool:
    return all(os.path.exists(asset(m, s)) for m in ("african_head", "diablo3_pose")
               for s in (".obj", "_diffuse.tga", "_nm_tangent.tga"))


def build() -> bool:
    """Build oracle/_ref (the reference's draw path headless, and the copies of its bundled
    assets) from the read-only reference sources when they are present."""
    if not have_reference():
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "assets", f"REF={REF_DIR}"], check=True)
    return available()


def _tex_bytes(tex) -> bytes:
    if tex is None:
        return struct.pack("<iii", 0, 0, 0)
    return struct.pack("<iii", tex.w, tex.h, tex.bpp) + np.ascontiguousarray(tex.data).tobytes()


def write_job(path: str, frame, obj_path: str, shader: int | None = None) -> None:
    sw, sh = frame.shadow_size
    shader = frame.shader if shader is None else shader
    with open(path, "wb") as f:
        f.write(b"HSRJOB1\0")
        f.write(struct.pack("<iiiii", frame.width, frame.height, sw, sh, shader))
        f.write(struct.pack("<ff", frame.clear_depth, frame.shadow_clear_depth))
        f.write(bytes(frame.clear_rgba) + bytes(frame.shadow_clear_rgba))
        f.write(np.ascontiguousarray(frame.sd).tobytes())
        f.write(_tex_bytes(frame.diffuse))
        f.write(_tex_bytes(frame.normal))
        p = obj_path.encode()
        f.write(struct.pack("<i", len(p)) + p)


def read_out(path: str) -> dict:
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"HSROUT1\0", "bad harness output"
    off = 8
    (has_shadow,) = struct.unpack_from("<i", data, off)
    off += 4
    out = {}
    for name in ["main"] + (["shadow"] if has_shadow else []):
        w, h = struct.unpack_from("<ii", data, off)
        off += 8
        depth = np.frombuffer(data, np.float32, w * h, off).reshape(h, w).copy()
        off += 4 * w * h
        color = np.frombuffer(data, np.uint8, w * h * 4, off).reshape(h, w, 4).copy()
        off += 4 * w * h
        out[name] = {"depth": depth, "color": color}
    return out


def run(frame, shader: int | None = None, obj_mesh=None, workdir: str | None = None, obj_path: str | None = None,
        harness: str = HARNESS) -> dict:
    """Render one frame with the reference.  ``obj_mesh`` overrides the mesh written to
    the OBJ (used for the per-face-uv prim-id run); ``obj_path`` draws an existing OBJ file
    as Model::Model reads it (a bundled asset, with its own normals); ``harness`` is the
    binary that draws (SHIM_HOST_HARNESS: the drop-in shim in place of graphics.cpp)."""
    from hsr import scenes  # noqa: WPS433 (harness-side import)

    if obj_mesh is None and obj_path is None and (frame.shader if shader is None else shader) == scenes.FLAT:
        obj_mesh = scenes.prim_id_mesh(frame.mesh)  # FLAT == PrimIdShader on per-face uvs
    own = workdir is None
    wd = workdir or tempfile.mkdtemp(prefix="hsrref_")
    try:
        obj = obj_path or os.path.join(wd, "mesh.obj")
        if obj_path is None:
            scenes.write_obj(obj_mesh if obj_mesh is not None else frame.mesh, obj)
        job = os.path.join(wd, "job.bin")
        out = os.path.join(wd, "out.bin")
        write_job(job, frame, obj, shader)
        subprocess.run([harness, "draw", job, out], check=True, stderr=subprocess.DEVNULL)
        return read_out(out)
    finally:
        if own:
            for n in os.listdir(wd):
                os.unlink(os.path.join(wd, n))
            os.rmdir(wd)


def run_prim_ids(frame) -> dict:
    """Reference coverage/depth plus prim ids (face id + 1, 0 = untouched) per pass."""
    import dataclasses

    from hsr import scenes

    # ids are >= 1, so a black clear marks untouched pixels as 0 (depth does not depend on it)
    frame = dataclasses.replace(frame, clear_rgba=(0, 0, 0, 0), shadow_clear_rgba=(0, 0, 0, 0))
    res = run(frame, shader=8 if frame.shader == scenes.SHADOW else 7, obj_mesh=scenes.prim_id_mesh(frame.mesh))
    for v in res.values():
        c = v["color"].astype(np.uint32)
        v["prim"] = c[:, :, 0] | (c[:, :, 1] << 8) | (c[:, :, 2] << 16)
    return res


def time_frames(frame, frames: int, workdir: str | None = None) -> float:
    """Milliseconds per frame of the reference on one host core."""
    from hsr import scenes

    wd = workdir or tempfile.mkdtemp(prefix="hsrref_")
    obj = os.path.join(wd, "mesh.obj")
    scenes.write_obj(frame.mesh, obj)
    job = os.path.join(wd, "job.bin")
    write_job(job, frame, obj)
    r = subprocess.run([HARNESS, "time", job, str(frames)], check=True, capture_output=True, text=True)
    return float(r.stdout.strip())


def ref_matrices(eye, target, up, fovy, aspect, near, far, light, ortho) -> dict:
    """Matrices built by the reference's maths.cpp for the given parameters."""
    wd = tempfile.mkdtemp(prefix="hsrmat_")
    try:
        p = os.path.join(wd, "p.bin")
        o = os.path.join(wd, "o.bin")
        vals = list(eye) + list(target) + list(up) + [fovy, aspect, near, far] + list(light) + list(ortho)
        with open(p, "wb") as f:
            f.write(np.array(vals, np.float32).tobytes())
        subprocess.run([HARNESS, "mats", p, o], check=True)
        a = np.fromfile(o, np.float32)
        return {"view": a[0:16], "proj": a[16:32], "camera_vp": a[32:48], "light_vp": a[48:64],
                "model_I": a[64:80], "light_dir": a[80:83]}
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)


def ref_obj_corners(obj_path: str) -> np.ndarray:
    """Model::Model's parse read per face corner in draw order: (nfaces, 3, 8) float32 =
    vert (3), uv (2), normal (3) as Model::normal returns it during the first draw."""
    wd = tempfile.mkdtemp(prefix="hsrobj_")
    try:
        o = os.path.join(wd, "o.bin")
        subprocess.run([HARNESS, "obj", obj_path, o], check=True, stderr=subprocess.DEVNULL)
        data = open(o, "rb").read()
        (nf,) = struct.unpack_from("<i", data, 0)
        return np.frombuffer(data, np.float32, nf * 24, 4).reshape(nf, 3, 8).copy()
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)


def ref_tga_read(tga_path: str, model_flip: bool) -> np.ndarray:
    """TGAImage::read_tga_file (+ Model::load_texture's flip): (h, w, bytespp) uint8."""
    wd = tempfile.mkdtemp(prefix="hsrtga_")
    try:
        o = os.path.join(wd, "o.bin")
        subprocess.run([HARNESS, "tga", tga_path, "1" if model_flip else "0", o], check=True, stderr=subprocess.DEVNULL)
        data = open(o, "rb").read()
        w, h, bpp = struct.unpack_from("<iii", data, 0)
        return np.frombuffer(data, np.uint8, w * h * bpp, 12).reshape(h, w, bpp).copy()
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)


def ref_tga_write(img: np.ndarray, rle: bool) -> bytes:
    """The bytes TGAImage::write_tga_file writes for an (h, w, bytespp) uint8 buffer."""
    wd = tempfile.mkdtemp(prefix="hsrtgaw_")
    try:
        i = os.path.join(wd, "i.bin")
        o = os.path.join(wd, "o.tga")
        h, w, bpp = img.shape
        with open(i, "wb") as f:
            f.write(struct.pack("<iii", w, h, bpp) + np.ascontiguousarray(img, np.uint8).tobytes())
        subprocess.run([HARNESS, "tgawrite", i, "1" if rle else "0", o], check=True, stderr=subprocess.DEVNULL)
        return open(o, "rb").read()
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)


def ref_uniforms(position, rotation_deg, scale, eye, target, light, width: int, height: int) -> dict:
    """GameObject::GetModelMatrix, its inverse, and DrawModel::draw's matrices and light
    direction from the reference (camera.cpp, maths.cpp, scene.h:55-71)."""
    wd = tempfile.mkdtemp(prefix="hsruni_")
    try:
        p = os.path.join(wd, "p.bin")
        o = os.path.join(wd, "o.bin")
        vals = list(position) + list(rotation_deg) + list(scale) + list(eye) + list(target) + list(light)
        with open(p, "wb") as f:
            f.write(np.array(vals, np.float32).tobytes() + struct.pack("<ii", width, height))
        subprocess.run([HARNESS, "uniforms", p, o], check=True)
        a = np.fromfile(o, np.float32)
        names = ["model", "model_I", "view", "proj", "light_vp", "camera_vp"]
        out = {n: a[16 * k:16 * (k + 1)] for k, n in enumerate(names)}
        out["light_dir"] = a[96:99]
        return out
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)


def ref_camera(cases: np.ndarray) -> np.ndarray:
    """Camera::update_transform (camera.cpp:63-70) of the reference for each row of `cases`
    (position[3], target[3], orbit[2], pan[2], dolly): rows of new position[3], target[3]."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 11)
    wd = tempfile.mkdtemp(prefix="hsrcam_")
    try:
        p = os.path.join(wd, "c.bin")
        o = os.path.join(wd, "o.bin")
        with open(p, "wb") as f:
            f.write(struct.pack("<i", len(cases)) + cases.tobytes())
        subprocess.run([HARNESS, "camera", p, o], check=True)
        return np.fromfile(o, np.float32).reshape(-1, 6)
    finally:
        for n in os.listdir(wd):
            os.unlink(os.path.join(wd, n))
        os.rmdir(wd)
