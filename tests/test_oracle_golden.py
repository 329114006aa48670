"""CPU: the oracle restatement against the reference's own outputs (golden fixtures), and
the host uniform builder against the reference's matrix builders."""
import os

import numpy as np
import pytest

import golden_io
import oracle
from hsr import uniforms as U


@pytest.mark.parametrize("name", golden_io.names())
def test_oracle_matches_reference(name):
    frame, exp = golden_io.load(name)
    out = oracle.render_frame(frame)
    for k, e in exp.items():
        got = {"depth": out[k].depth, "color": out[k].color, "prim": out[k].prim}
        golden_io.assert_pass(got, e, k, name)


def test_oracle_built_without_contraction():
    assert oracle.lib().hsro_no_contraction() == 1


def test_uniform_builder_matches_reference_bits():
    rows = np.load(os.path.join(golden_io.GOLDEN, "matrices.npy"))
    for r in rows:
        eye, (w, h) = tuple(float(x) for x in r[0:3]), (int(r[3]), int(r[4]))
        sd = U.shader_data(eye, w, h)
        exp = {"view_matrix": r[5:21], "projection_matrix": r[21:37], "camera_vp_matrix": r[37:53],
               "light_vp_matrix": r[53:69], "model_matrix_I": r[69:85], "light_dir": r[85:88]}
        for k, v in exp.items():
            got = np.asarray(sd[k], np.float32).reshape(-1)
            assert (got.view(np.uint32) == v.view(np.uint32)).all(), (eye, k)


def test_prim_ids_are_faces_plus_one():
    frame, exp = golden_io.load("soup_ties_12k")
    prim = exp["main"]["prim"]
    assert prim.max() <= frame.mesh.nfaces and (prim > 0).sum() > 0


def test_toon_single_precision_thresholds():
    """The device Toon shader compares the float intensity against the largest float not above
    each double constant of IShader.cpp:30-39; (double)f > c holds exactly when f > that float."""
    import re

    src = open(os.path.join(os.path.dirname(golden_io.GOLDEN), "..", "hana-softwarerenderer_gb300", "csrc",
                            "hsr_device.cuh")).read()
    found = re.findall(r"intensity > (0x[0-9a-f.]+p-\d)f\) intensity = [^;]+;\s+// (\.\d\d)", src)
    assert [c for _, c in found] == [".85", ".60", ".45", ".30", ".15"]
    for h, c in found:
        f = np.float32(float.fromhex(h))
        assert float(f) == float.fromhex(h)
        assert float(f) <= float(c) < float(np.nextafter(f, np.float32(1)))
