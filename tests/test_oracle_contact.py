"""The oracle's query::contact against the reference's known answers (CPU only)."""
import numpy as np
import pytest

from tests import _contact_cases as CC


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_cuboid_cuboid_epa(oracle_lib, prec):
    s, pairs, c = CC.cuboid_epa()
    has, out, st = oracle_lib.contacts(s, pairs, c["prediction"], precision=prec, threads=1)
    assert has.all()
    for k, case in enumerate(c["cases"]):
        assert out[k, 12] == case["expect_dist"] if prec == "f32" else abs(out[k, 12] - case["expect_dist"]) < 1e-6
        np.testing.assert_array_equal(out[k, 6:9], np.array(case["expect_normal1"], out.dtype))
    assert st["epa_calls"] == 2


def test_triangle_touch(oracle_lib):
    s, pairs, c = CC.triangle_touch()
    has, out, _ = oracle_lib.contacts(s, pairs, c["prediction"], threads=1)
    assert has[0] == 1
    assert abs(out[0, 1] - c["expect_point1_y"]) <= c["tolerance"]
    assert abs(out[0, 0] - c["expect_point1_x"]) <= c["tolerance"]


def test_ball_ball_prediction(oracle_lib):
    s, pairs, c = CC.ball_ball()
    for case in c["cases"]:
        has, out, _ = oracle_lib.contacts(s, pairs, case["prediction"], threads=1)
        if case["expect"] is None:
            assert has[0] == 0
        else:
            assert has[0] == 1 and 0 < out[0, 12] <= case["prediction"]


def test_ball_cuboid(oracle_lib):
    s, pairs, c = CC.ball_cuboid()
    has, out, _ = oracle_lib.contacts(s, pairs, c["prediction"], threads=1)
    assert has[0] == 1 and out[0, 12] <= 0
    assert has[1] == 1 and out[1, 12] >= 0
    assert has[2] == 0


def test_f32_close_to_f64_on_random_hulls(oracle_lib):
    from parry_gb300 import workloads as W
    s, pairs = W.hull_pairs(400, seed=3)
    h32, o32, _ = oracle_lib.contacts(s, pairs, 0.0, precision="f32")
    h64, o64, _ = oracle_lib.contacts(s, pairs, 0.0, precision="f64")
    same = h32 == h64
    assert same.mean() > 0.99
    both = (h32 == 1) & (h64 == 1)
    assert np.quantile(np.abs(o32[both, 12] - o64[both, 12]), 0.99) < 1e-4
