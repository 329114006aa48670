"""CPU: the asset readers and writers of the C ABI (hsr_obj_read, hsr_tga_read, hsr_tga_write)
— no device needed.

Against the reference: where its sources and bundled assets are present (this container),
Model::Model and TGAImage, compiled headless in oracle/_ref, parse the same files and the
results must match bit for bit; TGAImage::write_tga_file must write the same bytes.
Everywhere: exact round trips of synthetic files in every layout the reference reads.
"""
import os

import numpy as np
import pytest

import hsr
import refjob
import tga_files
from hsr import scenes

ASSETS = os.path.join(refjob.REF_DIR, "assets")
HAVE_REF = refjob.available() and os.path.isdir(ASSETS)
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources / assets not present on this host")


def ref_normalize_sequence(nrm: np.ndarray, faces: np.ndarray, earlier: int = 0) -> np.ndarray:
    """Per-corner normals of a draw after `earlier` others: Model::normal normalises the
    stored normal in place on every read (model.cpp:108-111, vector.h:41-42), faces in
    order, corners 0..2, every corner once per draw."""
    stored = nrm.astype(np.float32).copy()
    out = np.empty((faces.shape[0], 3, 3), np.float32)
    for _ in range(earlier + 1):
        for i in range(faces.shape[0]):
            for j in range(3):
                n = stored[faces[i, j, 2]]
                ln = np.sqrt(np.float32(n[0] * n[0] + n[1] * n[1]) + np.float32(n[2] * n[2]), dtype=np.float32)
                n *= np.float32(1.0) / ln
                out[i, j] = n
    return out


def test_obj_round_trip(tmp_path):
    m = scenes.sphere_mesh(3, displace=0.05, seed=4)
    p = tmp_path / "m.obj"
    scenes.write_obj(m, str(p))
    pos, nrm, uv, faces = hsr.obj_read(str(p))
    assert np.array_equal(pos.view(np.uint32), m.pos.view(np.uint32))
    assert np.array_equal(nrm.view(np.uint32), m.nrm.view(np.uint32))
    assert np.array_equal(uv.view(np.uint32), m.uv.view(np.uint32))
    assert np.array_equal(faces, m.faces)


@pytest.mark.parametrize("earlier", [0, 1, 3])
def test_obj_corner_normals(tmp_path, earlier):
    rng = np.random.default_rng(2)
    m = scenes.sphere_mesh(2, seed=1)
    nrm = (m.nrm * rng.uniform(0.5, 2.0, (len(m.nrm), 1))).astype(np.float32)  # not unit length
    m = scenes.Mesh(m.pos, nrm, m.uv, m.faces)
    p = tmp_path / "m.obj"
    scenes.write_obj(m, str(p))
    pos, cn, uv, faces = hsr.obj_read(str(p), hsr.OBJ_CORNER_NORMALS | hsr.obj_earlier_draws(earlier))
    assert cn.shape == (3 * m.nfaces, 3)
    assert np.array_equal(faces[:, :, 2].reshape(-1), np.arange(3 * m.nfaces))
    want = ref_normalize_sequence(nrm, m.faces, earlier).reshape(-1, 3)
    assert np.array_equal(cn.view(np.uint32), want.view(np.uint32))


def test_obj_quads_draw_their_first_three_corners(tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\n"
                 "f 1/1/1 2/1/1 3/1/1 4/1/1\r\nf 1/1/1 3/1/1 4/1/1\n")
    pos, nrm, uv, faces = hsr.obj_read(str(p))
    assert faces.shape == (2, 3, 3)
    assert faces[0, :, 0].tolist() == [0, 1, 2] and faces[1, :, 0].tolist() == [0, 2, 3]


def test_obj_errors_are_status_codes(tmp_path):
    with pytest.raises(hsr.HsrError):
        hsr.obj_read(str(tmp_path / "missing.obj"))
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 1/1/1\n")  # index past the vertices
    with pytest.raises(hsr.HsrError):
        hsr.obj_read(str(p))
    p.write_text("v 0 0 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 1/1/1\n")  # fewer than three corners
    with pytest.raises(hsr.HsrError):
        hsr.obj_read(str(p))


@pytest.mark.parametrize("bpp", [1, 3, 4])
@pytest.mark.parametrize("rle", [False, True])
@pytest.mark.parametrize("top_left,right_left", [(True, False), (False, False), (False, True)])
def test_tga_read_layouts(tmp_path, bpp, rle, top_left, right_left):
    img = tga_files.runs_image(37, 53, bpp, seed=bpp * 7 + rle)
    p = tmp_path / "t.tga"
    p.write_bytes(tga_files.encode(img, rle, top_left, right_left))
    got = hsr.tga_read(str(p))
    assert np.array_equal(got, img)
    # Model::load_texture flips once more
    assert np.array_equal(hsr.tga_read(str(p), hsr.TGA_MODEL_FLIP), img[::-1])


@pytest.mark.parametrize("bpp", [1, 3, 4])
@pytest.mark.parametrize("rle", [False, True])
def test_tga_write_read_round_trip(tmp_path, bpp, rle):
    img = tga_files.runs_image(41, 29, bpp, seed=bpp + 11 * rle)
    p = tmp_path / "w.tga"
    hsr.tga_write(str(p), img, rle)
    assert np.array_equal(hsr.tga_read(str(p)), img)


def test_tga_errors_are_status_codes(tmp_path):
    p = tmp_path / "bad.tga"
    p.write_bytes(b"\0" * 10)
    with pytest.raises(hsr.HsrError):
        hsr.tga_read(str(p))
    img = tga_files.runs_image(8, 8, 3, seed=1)
    data = tga_files.encode(img, True)
    p.write_bytes(data[:-5])  # truncated run-length data
    with pytest.raises(hsr.HsrError):
        hsr.tga_read(str(p))


# ---- against the reference's own parsers and writer -----------------------------------------
@needs_ref
@pytest.mark.parametrize("asset", ["african_head/african_head.obj", "diablo3_pose/diablo3_pose.obj"])
def test_obj_matches_reference_model(asset):
    path = os.path.join(ASSETS, asset)
    want = refjob.ref_obj_corners(path)
    pos, nrm, uv, faces = hsr.obj_read(path, hsr.OBJ_CORNER_NORMALS)
    got = np.concatenate([pos[faces[:, :, 0]], uv[faces[:, :, 1]], nrm[faces[:, :, 2]]], axis=2)
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@needs_ref
@pytest.mark.parametrize("asset", ["african_head/african_head_diffuse.tga", "african_head/african_head_nm_tangent.tga",
                                   "african_head/african_head_spec.tga", "diablo3_pose/diablo3_pose_diffuse.tga",
                                   "diablo3_pose/diablo3_pose_nm_tangent.tga"])
def test_tga_matches_reference_reader(asset):
    path = os.path.join(ASSETS, asset)
    for flip in (False, True):
        want = refjob.ref_tga_read(path, flip)
        got = hsr.tga_read(path, hsr.TGA_MODEL_FLIP if flip else 0)
        assert np.array_equal(got, want)


@needs_ref
@pytest.mark.parametrize("bpp", [1, 3, 4])
@pytest.mark.parametrize("rle", [False, True])
def test_tga_layouts_match_reference_reader(tmp_path, bpp, rle):
    img = tga_files.runs_image(23, 31, bpp, seed=5 * bpp + rle)
    for tl, rl in ((True, False), (False, False), (False, True)):
        p = tmp_path / "t.tga"
        p.write_bytes(tga_files.encode(img, rle, tl, rl))
        assert np.array_equal(hsr.tga_read(str(p)), refjob.ref_tga_read(str(p), False))


@needs_ref
@pytest.mark.parametrize("bpp", [1, 3, 4])
@pytest.mark.parametrize("rle", [False, True])
def test_tga_writer_bytes_match_reference(tmp_path, bpp, rle):
    img = tga_files.runs_image(45, 67, bpp, seed=3 * bpp + rle)
    p = tmp_path / "w.tga"
    hsr.tga_write(str(p), img, rle)
    assert p.read_bytes() == refjob.ref_tga_write(img, rle)
