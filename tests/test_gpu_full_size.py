"""Parity at the full sizes of the measured workloads, through the C ABI, against the oracle's f32
restatement of parry3d on the same inputs:

- batched uneven GJK/EPA: all 1,048,576 hull pairs (8-256 vertices), has-contact decisions and the
  GJK / EPA iteration counts identical, points, normals and depth within 1e-5;
- learned warm start: the same 1,048,576 pairs started from the network's predicted directions,
  against the oracle given the same `init_dir`s (contact_support_map_support_map_with_params);
- per-frame pipeline: 262,144 shapes and 4,194,304 rays, 3 frames: poses, pair sets, manifold
  records and ray hits bit-exact; and the same shapes with the network seeding new pairs, against
  the oracle's frame loop given the network's directions.
"""
import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5
FULL_PAIRS = 1 << 20


def _compare_contacts(has, out, st, ho, oo, sto, what):
    np.testing.assert_array_equal(has, ho, err_msg=f"has_contact differs ({what})")
    m = ho == 1
    np.testing.assert_allclose(out[m], oo[m], rtol=TOL, atol=TOL, err_msg=what)
    assert st["gjk_iters"] == sto["gjk_iters"], what
    assert st["epa_iters"] == sto["epa_iters"], what
    assert st["epa_calls"] == sto["epa_calls"], what


@pytest.fixture(scope="module")
def hull_pairs_full():
    return W.hull_pairs(FULL_PAIRS)


@pytest.fixture(scope="module")
def hull_pairs_oracle(oracle_lib, hull_pairs_full):
    s, pairs = hull_pairs_full
    return oracle_lib.contacts(s, pairs, 0.0)


@pytest.mark.parametrize("warp_cost,epa_inline", [(0, 0), (4096, 1), (160, 2), (2, 0)])
def test_uneven_hull_pairs_full_size(oracle_lib, hull_pairs_full, hull_pairs_oracle, warp_cost, epa_inline):
    """The library defaults (0, 0); one thread per pair with EPA right after GJK (4096, 1); the dearer
    pairs one warp each (160); every pair one warp (2)."""
    s, pairs = hull_pairs_full
    ctx = pg.Context(0, contact_warp_cost=warp_cost, contact_epa_inline=epa_inline)
    try:
        has, out, st = pg.contacts(ctx, s, pairs, 0.0, want_stats=True)
    finally:
        ctx.close()
    ho, oo, sto = hull_pairs_oracle
    _compare_contacts(has, out, st, ho, oo, sto, f"1,048,576 uneven hull pairs, warp cost {warp_cost}")
    assert 0.3 < ho.mean() < 0.9
    print(f"\n{int(ho.sum())} contacts; GJK {st['gjk_iters'] / FULL_PAIRS:.3f} and EPA {st['epa_iters'] / FULL_PAIRS:.3f} "
          f"iterations per pair, {st['epa_calls']} EPA calls, identical to the oracle")


def test_learned_warm_start_full_size(gpu_ctx, oracle_lib, hull_pairs_full):
    """The learned run's answers against the oracle started from the same predicted directions."""
    import torch
    s_tr, p_tr = W.hull_pairs(65536, seed=0x51AB1E)
    mlp = pg.WarmStartMLP(gpu_ctx, seed=7)
    labels = np.zeros((len(p_tr), 3), np.float32)
    pg.contacts(gpu_ctx, s_tr, p_tr, 0.0, final_dirs=labels)
    labels /= np.maximum(np.linalg.norm(labels, axis=1, keepdims=True), 1e-12)
    f_tr = torch.from_numpy(np.ascontiguousarray(mlp.features(s_tr, p_tr))).cuda()
    mlp.train(f_tr, torch.from_numpy(labels).cuda(), epochs=2, batch=8192, lr=2e-3)
    s, pairs = hull_pairs_full
    init = np.ascontiguousarray(mlp.predict(mlp.features(s, pairs)), np.float32)
    assert init.shape == (FULL_PAIRS, 3) and np.isfinite(init).all()
    has, out, st = pg.contacts(gpu_ctx, s, pairs, 0.0, init_dirs=init, want_stats=True)
    ho, oo, sto = oracle_lib.contacts(s, pairs, 0.0, init_dirs=init)
    _compare_contacts(has, out, st, ho, oo, sto, "learned init_dir on 1,048,576 hull pairs")


def test_frame_pipeline_full_size(gpu_ctx, oracle_lib):
    """262,144 shapes (ball / cuboid / capsule / hull, 25 % each) in an 800-wide cube and 4,194,304
    rays: three frames of integrate, AABBs, refit, pairs, manifolds and rays against the oracle's
    frame loop. The pair set and manifold records depend on every earlier frame, so the last frame
    checks the whole chain."""
    import torch
    from parry_gb300 import manifold as M
    frames, pred, dt, max_toi = 3, 0.1, 1.0 / 60.0, 100.0
    t, prm, pos, pool, poly, vel, rays = W.frame_scene(262144, 4194304, 400.0)
    shapes = pg.ShapeSet.from_arrays(t, prm, pos, pool, poly)
    sc = pg.Scene(gpu_ctx, shapes, vel, pred, 1 << 20)
    sc.set_rays(torch.from_numpy(rays).cuda(), max_toi)
    sc.step(dt, frames, use_graph=True)
    frame, npairs = sc.info()
    got = sc.read()
    sc.close()
    want = oracle_lib.scene_frames(shapes, vel, pred, dt, frames, rays=rays, max_toi=max_toi)
    assert frame == frames
    np.testing.assert_array_equal(got["poses"], want["poses"])
    order = np.lexsort((got["pairs"][:, 1], got["pairs"][:, 0]))
    assert npairs == len(want["pairs"]) and npairs > 10000
    np.testing.assert_array_equal(got["pairs"][order], want["pairs"])
    gw = M.as_words(got["manifolds"])[order]
    ww = want["manifolds"]
    np.testing.assert_array_equal(gw[:, :8], ww[:, :8])
    n = ww[:, 0].astype(np.int64)
    valid = np.arange(M.MAX_POINTS)[None, :] < n[:, None]
    np.testing.assert_array_equal(gw[:, 8:].reshape(len(gw), M.MAX_POINTS, 10)[valid],
                                  ww[:, 8:].reshape(len(ww), M.MAX_POINTS, 10)[valid])
    np.testing.assert_array_equal(got["ray_part"], want["ray_part"])
    np.testing.assert_array_equal(got["ray_toi"], want["ray_toi"])
    np.testing.assert_array_equal(got["ray_normal"], want["ray_normal"])
    print(f"\n{npairs} pairs, {int((n > 0).sum())} with contact points, "
          f"{int((want['ray_part'] != pg.NO_HIT).sum())} ray hits: identical to the oracle")


def test_frame_pipeline_learned_seeding_full_size(gpu_ctx, oracle_lib):
    """The same 262,144 shapes for 3 graph frames with the network seeding the pairs that hold no
    cached normal: poses, pair sets and manifold records against the oracle's frame loop given the
    network's directions for each frame's pairs (rays do not depend on the seeding and are left out)."""
    from parry_gb300 import manifold as M
    frames, pred, dt = 3, 0.1, 1.0 / 60.0
    t, prm, pos, pool, poly, vel, _ = W.frame_scene(262144, 16, 400.0)
    shapes = pg.ShapeSet.from_arrays(t, prm, pos, pool, poly)
    mlp = pg.WarmStartMLP(gpu_ctx, seed=5)
    sc = pg.Scene(gpu_ctx, shapes, vel, pred, 1 << 20)
    sc.set_mlp(mlp)
    sc.step(dt, frames, use_graph=True)
    got = sc.read()
    seeded = sc.stats()["seeded_pairs"]
    sc.close()
    want = oracle_lib.scene_frames(shapes, vel, pred, dt, frames,
                                   dirs_fn=lambda s, p: mlp.predict(mlp.features(s, p)))
    np.testing.assert_array_equal(got["poses"], want["poses"])
    order = np.lexsort((got["pairs"][:, 1], got["pairs"][:, 0]))
    np.testing.assert_array_equal(got["pairs"][order], want["pairs"])
    gw = M.as_words(got["manifolds"])[order]
    ww = want["manifolds"]
    np.testing.assert_array_equal(gw[:, :8], ww[:, :8])
    n = ww[:, 0].astype(np.int64)
    valid = np.arange(M.MAX_POINTS)[None, :] < n[:, None]
    np.testing.assert_array_equal(gw[:, 8:].reshape(len(gw), M.MAX_POINTS, 10)[valid],
                                  ww[:, 8:].reshape(len(ww), M.MAX_POINTS, 10)[valid])
    assert seeded > 0
    print(f"\n{len(ww)} pairs, {seeded} seeded in the last frame: identical to the oracle")
