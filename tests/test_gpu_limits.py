"""GPU: targets at the size limits of the C ABI against the oracle.

hsr_target_create accepts 1..32768 pixels a side.  These draws put triangles across the whole
extent of the widest (32768 x 256) and tallest (256 x 32768) targets — pixel coordinates up to
32767 in the records' 16-bit ranges, tile rows 4096 tiles long — and over a 16384 x 8192 target
(134M pixels, half a million 16x16 tiles through the scan, the scatter's clear and the raster)
with two triangles that together cover the whole target (clipped, then split into sub-records by
k_big).
Tolerances as in test_gpu_parity: depth, prim ids and alpha bit for bit, RGB within 1 LSB (the
flat test shader's colour is exact).
"""
import numpy as np
import pytest

import golden_io
import oracle
from hsr import frame as hframe
from hsr import scenes

pytestmark = pytest.mark.gpu


def _render(frame):
    g = hframe.GpuFrame(frame)
    try:
        g.render(batched=True)
        return g.download()
    finally:
        g.release()


def _check(frame, label):
    got = _render(frame)
    out = oracle.render_frame(frame)
    for k, v in out.items():
        golden_io.assert_pass(got[k], {"depth": v.depth, "color": v.color, "prim": v.prim}, k, label)
    return got


def _with_covering_triangles(frame, depths):
    """The soup plus, drawn after it, two triangles per depth whose union covers the target."""
    m = frame.mesh
    n0 = len(m.pos)
    extra = []
    for z in depths:
        extra += [(-1.5, -1.5, z), (1.5, -1.5, z), (1.5, 1.5, z), (-1.5, 1.5, z)]
    pos = np.concatenate([m.pos, np.asarray(extra, np.float32)])
    quads = []
    for q in range(len(depths)):
        b = n0 + 4 * q
        quads += [(b, b + 1, b + 2), (b, b + 2, b + 3)]
    faces = np.zeros((m.nfaces + len(quads), 3, 3), np.int32)
    faces[: m.nfaces] = m.faces
    faces[m.nfaces:, :, 0] = np.asarray(quads, np.int32)
    frame.mesh = scenes.Mesh(pos, m.nrm, m.uv, faces)
    return frame


@pytest.mark.parametrize("w,h", [(32768, 256), (256, 32768)])
def test_widest_and_tallest_targets_vs_oracle(gpu, w, h):
    frame = scenes.soup_frame(60_000, w, h, seed=23, median_edge_px=3.0)
    got = _check(frame, f"soup {w}x{h}")
    # triangles reach both ends of the long side
    drawn = got["main"]["prim"] > 0
    along = drawn.any(axis=0) if w > h else drawn.any(axis=1)
    assert along[:64].any() and along[-64:].any()


def test_16384x8192_target_with_covering_triangles_vs_oracle(gpu):
    frame = _with_covering_triangles(scenes.soup_frame(200_000, 16384, 8192, seed=29, median_edge_px=6.0), [0.6])
    got = _check(frame, "soup 16384x8192 + covering triangles")
    assert (got["main"]["prim"] > 0).all()  # the covering triangles reach every pixel
