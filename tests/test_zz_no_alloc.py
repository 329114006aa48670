"""GPU: hsr_draw_noalloc, the draw entry point for callers that cannot allocate while they
draw (work captured into a CUDA graph, real-time loops, fixed memory budgets).

It must produce what hsr_draw produces — depth and prim ids bit for bit, colour within the
1 LSB the parity tests allow — on two calls in a row, since every call reuses the same
fixed scratch array and must clear whatever has to start from zero.  This file is named to
be collected last, and it initialises the library itself so it also passes alone in a
fresh process.
"""
import numpy as np
import pytest

import hsr
from hsr import frame as hframe
from hsr import scenes

pytestmark = pytest.mark.gpu

COLOR_TOL = 1


def _same(a, b):
    for name in ("depth", "prim"):
        assert np.array_equal(a[name].view(np.uint32), b[name].view(np.uint32)), name
    dc = np.abs(a["color"].astype(np.int32) - b["color"].astype(np.int32)).max()
    assert dc <= COLOR_TOL, dc


def test_noalloc_draw_matches_draw_twice_in_a_row():
    hsr.init(0)
    # a shadowed frame: the shadow pass, then the main pass that samples it
    fr = scenes.displaced_frame(5, 320, 240, shadow=256, tex_size=128, seed=3)
    g = hframe.GpuFrame(fr)
    try:
        for d in g.descs:
            hsr.draw(d)
        want = g.download()
        for _ in range(2):
            # wipe the targets so nothing carries over from the previous call
            g.main.clear((7, 7, 7, 7), 0.0)
            g.shadow.clear((7, 7, 7, 7), 0.0)
            for d in g.descs:
                hsr.draw_noalloc(d)
            got = g.download()
            for k in want:
                _same(got[k], want[k])
    finally:
        g.release()


def test_noalloc_draw_refuses_oversized_draws():
    hsr.init(0)
    fr = scenes.soup_frame(800_000, 1920, 1080, seed=5)
    g = hframe.GpuFrame(fr)
    try:
        with pytest.raises(hsr.HsrError) as e:
            hsr.draw_noalloc(g.descs[0])
        assert e.value.code == hsr.ERR_INVALID_ARG
    finally:
        g.release()
