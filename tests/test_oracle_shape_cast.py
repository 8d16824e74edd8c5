"""The oracle's restatement of query::cast_shapes (linear shape casting): the reference's own
time-of-impact tests, and properties on random convex pairs (after moving both shapes by toi x
velocity they touch; swapping the pair keeps the toi; f32 agrees with f64)."""
import numpy as np
import pytest

from parry_gb300 import workloads as W
from parry_gb300.shapes import ShapeSet
from tests import _contact_cases as CC


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reference_toi_cases(oracle_lib, prec):
    s, pairs, vels, expect = CC.toi_cases()
    status, out, _ = oracle_lib.cast_shapes(s, pairs, vels, precision=prec, threads=1)
    if prec == "f32":
        CC.check_toi(status, out, expect)
    else:
        for k, e in enumerate(expect):
            assert (status[k] == 255) == (e[0] == "none")
            if e[0] in ("toi", "toi_rel"):
                assert abs(out[k, 0] - e[1]) <= 1e-6


def _random_casts(n, seed):
    s, pairs = W.mixed_contact_pairs(n, seed=seed)
    t, prm, pos, pool = s.arrays()
    pos = pos.copy()
    rng = np.random.default_rng(seed)
    # separate the pairs and send the second shape back towards the first
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos[1::2, 4:7] += 6.0 * d
    vels = np.zeros((2 * n, 3), np.float32)
    vels[1::2] = -d * rng.uniform(0.5, 2.0, (n, 1)).astype(np.float32)
    return ShapeSet.from_arrays(t, prm, pos, pool), pairs, vels


def test_hits_touch_after_moving(oracle_lib):
    s, pairs, vels = _random_casts(2000, 5)
    status, out, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0)
    conv = status == 1
    assert conv.mean() > 0.5
    t, prm, pos, pool = s.arrays()
    moved = pos.copy()
    k = np.nonzero(conv)[0]
    for j in (0, 1):
        idx = pairs[k, j]
        moved[idx, 4:7] += vels[idx] * out[k, 0:1]
    s2 = ShapeSet.from_arrays(t, prm, moved, pool)
    has, c, _ = oracle_lib.contacts(s2, pairs[k], 0.05)
    # the GJK ray cast stops within its relative tolerance (sqrt of eps_tol, about 1e-3)
    assert has.mean() > 0.995
    assert np.quantile(np.abs(c[has == 1, 12]), 0.99) < 2e-3


def test_swapped_pair_same_toi(oracle_lib):
    s, pairs, vels = _random_casts(2000, 6)
    st1, o1, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0)
    st2, o2, _ = oracle_lib.cast_shapes(s, pairs[:, ::-1].copy(), vels, max_toi=100.0)
    both = (st1 == 1) & (st2 == 1)
    assert (st1 == 255).tolist() == (st2 == 255).tolist() or np.mean((st1 == 255) == (st2 == 255)) > 0.995
    err = np.abs(o1[both, 0] - o2[both, 0]) / np.maximum(np.abs(o2[both, 0]), 1e-3)
    assert np.quantile(err, 0.99) < 1e-3 and err.max() < 5e-3


def test_f32_close_to_f64(oracle_lib):
    s, pairs, vels = _random_casts(2000, 7)
    st32, o32, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0)
    st64, o64, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0, precision="f64")
    assert np.mean(st32 == st64) > 0.99
    both = (st32 == 1) & (st64 == 1)
    err = np.abs(o32[both, 0] - o64[both, 0]) / np.maximum(np.abs(o64[both, 0]), 1e-3)
    assert np.quantile(err, 0.99) < 1e-3 and err.max() < 5e-3


def test_options(oracle_lib):
    """target_distance stops earlier by that distance; max_toi rejects later hits; a pair already
    penetrating reports toi 0 with the contact geometry, or nothing when it separates and
    stop_at_penetration is off."""
    s, pairs, vels = _random_casts(500, 8)
    st0, o0, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0)
    st1, o1, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=100.0, target_distance=0.1)
    both = (st0 == 1) & (st1 == 1)
    assert both.sum() > 100 and (o1[both, 0] <= o0[both, 0] + 1e-6).all()
    stm, om, _ = oracle_lib.cast_shapes(s, pairs, vels, max_toi=2.0)
    assert ((stm != 255) <= (st0 != 255)).all() and (om[stm != 255, 0] <= 2.0).all()
    sp, pp = W.mixed_contact_pairs(300, seed=9)
    has, _, _ = oracle_lib.contacts(sp, pp, 0.0)
    v = np.zeros((600, 3), np.float32)
    v[1::2] = [0.0, 1.0, 0.0]
    stp, op, _ = oracle_lib.cast_shapes(sp, pp, v)
    assert (stp[has == 1] == 3).all() and (op[has == 1, 0] == 0).all()
