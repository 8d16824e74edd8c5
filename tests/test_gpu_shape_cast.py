"""Parity of the CUDA shape-casting path (query::cast_shapes through the C ABI) with the oracle's
f32 restatement: the reference's time-of-impact tests, and random ball / cuboid / capsule / hull
pairs (W.shape_cast_pairs) under every option, status identical and hit values within 1e-5."""
import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import workloads as W
from tests import _contact_cases as CC

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _compare(st, out, so, oo):
    np.testing.assert_array_equal(st, so)
    m = so != pg.CAST_NONE
    np.testing.assert_allclose(out[m], oo[m], rtol=TOL, atol=TOL)


def _casts(n, seed):
    return W.shape_cast_pairs(n, seed=seed)


def test_reference_toi_cases(gpu_ctx, oracle_lib):
    s, pairs, vels, expect = CC.toi_cases()
    st, out = pg.cast_shapes(gpu_ctx, s, pairs, vels)
    CC.check_toi(st, out, expect)
    so, oo, _ = oracle_lib.cast_shapes(s, pairs, vels)
    _compare(st, out, so, oo)


@pytest.mark.parametrize("opts", [{}, {"target_distance": 0.1}, {"max_toi": 2.0},
                                  {"stop_at_penetration": False}, {"compute_impact_geometry_on_penetration": False},
                                  {"stop_at_penetration": False, "target_distance": 0.05}])
def test_random_pairs_vs_oracle(gpu_ctx, oracle_lib, opts):
    s, pairs, vels = _casts(40_000, 31)
    kw = {"max_toi": 100.0, **opts}
    st, out, stats = pg.cast_shapes(gpu_ctx, s, pairs, vels, want_stats=True, **kw)
    so, oo, sto = oracle_lib.cast_shapes(s, pairs, vels, **kw)
    _compare(st, out, so, oo)
    assert stats["epa_calls"] == sto["epa_calls"] and stats["epa_iters"] == sto["epa_iters"]
    assert (st == 1).sum() > 1000


def test_penetrating_pairs_and_device_buffers(gpu_ctx, oracle_lib):
    """Pairs that already overlap (toi 0 with the contact geometry from GJK/EPA), through device
    buffers."""
    import torch
    s, pairs = W.mixed_contact_pairs(20_000, seed=41)
    rng = np.random.default_rng(41)
    vels = rng.normal(size=(40_000, 3)).astype(np.float32)
    so, oo, sto = oracle_lib.cast_shapes(s, pairs, vels)
    assert (so == 3).sum() > 5000 and sto["epa_calls"] > 1000
    t, prm, pos, pool = s.arrays()
    dev = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    st, out = pg.cast_shapes(gpu_ctx, dev, torch.from_numpy(pairs.view(np.int32)).cuda(), torch.from_numpy(vels).cuda())
    gpu_ctx.sync()
    _compare(st.cpu().numpy(), out.cpu().numpy(), so, oo)
