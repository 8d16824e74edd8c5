"""The oracle against the reference's own known answers (CPU only)."""
import json
from pathlib import Path

import numpy as np
import pytest

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_trimesh_culling_triangle(oracle_lib, prec):
    O = oracle_lib
    case = KA["trimesh_culling_triangle"]
    m = O.TriMesh(np.array(case["vertices"], np.float32), np.array(case["indices"], np.uint32), prec)
    rays = np.array([r["origin"] + r["dir"] for r in case["rays"]], np.float32)
    f, t, n = m.cast_rays_and_get_normal(rays, case["max_toi"], threads=1)
    for k, r in enumerate(case["rays"]):
        assert f[k] == r["expect_feature"], r["name"]
        assert t[k] == pytest.approx(r["expect_toi"], rel=1e-6), r["name"]
        np.testing.assert_allclose(n[k], r["expect_normal"], atol=1e-6)


def test_golden_fixture_reproduces(oracle_lib):
    """The committed terrain fixture is reproduced bit-exactly by the oracle built here."""
    O = oracle_lib
    g = np.load(Path(__file__).parent / "golden" / "terrain_small.npz")
    m = O.TriMesh(g["vertices"], g["indices"], "f32")
    f, t, n = m.cast_rays_and_get_normal(g["rays"], float(g["max_toi"]), threads=1)
    np.testing.assert_array_equal(f, g["feature_f32"])
    np.testing.assert_array_equal(t, g["toi_f32"])
    np.testing.assert_array_equal(n, g["normal_f32"])
    m64 = O.TriMesh(g["vertices"], g["indices"], "f64")
    f2, t2, _ = m64.cast_rays_and_get_normal(g["rays"], float(g["max_toi"]), threads=1)
    np.testing.assert_array_equal(f2, g["feature_f64"])
    np.testing.assert_array_equal(t2, g["toi_f64"])
