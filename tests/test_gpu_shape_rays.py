"""Parity of the CUDA shape-set (Compound) ray casts with the oracle: hit part indices identical,
toi and normals within 1e-5; the reference's known answers hold."""
import numpy as np
import pytest

import parry_gb300 as pg
from tests import _contact_cases as CC

pytestmark = pytest.mark.gpu
REL = 1e-5


def _compare(p, t, n, po, to, no, what=""):
    np.testing.assert_array_equal(p, po, err_msg=what)
    hit = po != pg.NO_HIT
    np.testing.assert_allclose(t[hit], to[hit], rtol=REL, atol=REL, err_msg=what)
    np.testing.assert_allclose(n[hit], no[hit], rtol=REL, atol=REL, err_msg=what)


def test_known_answers(gpu_ctx):
    s, rays, c = CC.cuboid_ray()
    comp = pg.Compound(gpu_ctx, s)
    p, t, n = comp.cast_rays_and_get_normal(rays, c["max_toi"], solid=c["solid"])
    assert p[0] == 0 and t[0] == c["expect_toi"]
    np.testing.assert_array_equal(n[0], np.array(c["expect_normal"], np.float32))
    s, c = CC.solid_ray_cast()
    comp = pg.Compound(gpu_ctx, s)
    for case in c["cases"]:
        p, t, _ = comp.cast_rays_and_get_normal(np.array([case["ray"]], np.float32), np.finfo(np.float32).max, solid=case["solid"])
        assert (p[0] == pg.NO_HIT) if case["expect_toi"] is None else (p[0] == 0 and t[0] == case["expect_toi"])


@pytest.mark.parametrize("solid", [True, False])
def test_mixed_scene_vs_oracle(gpu_ctx, oracle_lib, solid):
    s = CC.mixed_scene(3000, seed=9, extent=30.0)
    rng = np.random.default_rng(10)
    o = rng.uniform(-35, 35, (200_000, 3))
    d = rng.normal(size=(200_000, 3))
    rays = np.concatenate([o, d], 1).astype(np.float32)
    comp = pg.Compound(gpu_ctx, s)
    p, t, n = comp.cast_rays_and_get_normal(rays, 100.0, solid=solid)
    po, to, no = oracle_lib.Compound(s).cast_rays_and_get_normal(rays, 100.0, solid=solid)
    _compare(p, t, n, po, to, no, f"solid={solid}")
    assert (po != pg.NO_HIT).sum() > 10_000


def test_set_poses_refit(gpu_ctx, oracle_lib):
    s = CC.mixed_scene(500, seed=12, extent=15.0)
    comp = pg.Compound(gpu_ctx, s)
    t_, prm, pos, pool = s.arrays()
    pos2 = pos.copy()
    pos2[:, 4:7] += np.random.default_rng(3).uniform(-2, 2, (len(pos), 3)).astype(np.float32)
    comp.set_poses(pos2)
    s2 = pg.ShapeSet.from_arrays(t_, prm, pos2, pool)
    rng = np.random.default_rng(5)
    rays = np.concatenate([rng.uniform(-20, 20, (50_000, 3)), rng.normal(size=(50_000, 3))], 1).astype(np.float32)
    pose = np.array([0.1, -0.2, 0.05, 0.97, 1.0, 2.0, -1.0], np.float32)
    pose[:4] /= np.linalg.norm(pose[:4])
    p, t, n = comp.cast_rays_and_get_normal(rays, 60.0, pose=pose)
    po, to, no = oracle_lib.Compound(s2).cast_rays_and_get_normal(rays, 60.0, pose=pose)
    _compare(p, t, n, po, to, no, "after set_poses")


def test_candidate_overflow_falls_back_exactly(gpu_ctx, oracle_lib):
    """A row of capsules and hulls along every ray: the support-map candidates overflow the wavefront
    list (4 per ray + 1024), and the affected rays are recast by the single-kernel path."""
    O = oracle_lib
    s = pg.ShapeSet()
    rng = np.random.default_rng(5)
    pts = rng.normal(size=(24, 3))
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    for i in range(400):
        pose = (0.0, 0.0, 0.0, 1.0, 2.0 * i, 0.0, 0.0)
        if i % 2:
            s.add_capsule(0.4, 0.3, pose)
        else:
            s.add_convex(pts * 0.5, pose)
    n = 64
    o = np.stack([np.full(n, -5.0), rng.uniform(-0.2, 0.2, n), rng.uniform(-0.2, 0.2, n)], 1)
    d = np.tile([1.0, 0.0, 0.0], (n, 1)) + rng.normal(scale=1e-3, size=(n, 3))
    rays = np.concatenate([o, d], 1).astype(np.float32)
    comp = pg.Compound(gpu_ctx, s)
    for solid in (True, False):
        p, t, nn = comp.cast_rays_and_get_normal(rays, 1000.0, solid=solid)
        po, to, no = O.Compound(s).cast_rays_and_get_normal(rays, 1000.0, solid=solid)
        _compare(p, t, nn, po, to, no, f"solid={solid}")
        assert np.all(p != pg.NO_HIT)
