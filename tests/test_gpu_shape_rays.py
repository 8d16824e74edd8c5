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


def _grazing_rays(rng, n, centre, radial, along, offset, dist):
    """Rays passing the point centre + radial * offset (radial a unit vector) with a direction
    perpendicular to `radial` (tilted by `along`), starting `dist` before that point."""
    side = np.cross(radial, along)
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    tilt = rng.uniform(-0.5, 0.5, (n, 1))
    d = side + tilt * along
    d -= radial * np.sum(d * radial, axis=1, keepdims=True)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = centre + radial * offset[:, None]
    return np.concatenate([p - d * dist[:, None], d], 1).astype(np.float32)


@pytest.mark.parametrize("solid", [True, False])
def test_grazing_rays_match_oracle(gpu_ctx, oracle_lib, solid):
    """Rays grazing capsules and hulls, from just inside to 5 % outside their surfaces. On rounded
    shapes parry's GJK ray cast reports hits a little outside the surface; the pre-tests that drop
    candidates before the GJK ray cast (local box, capsule axis distance) must not drop any of them,
    so every answer equals the oracle's."""
    from parry_gb300.shapes import CAPSULE, CONVEX
    rng = np.random.default_rng(21 + solid)
    s = CC.mixed_scene(400, seed=23, extent=40.0)
    t, prm, pos, pool = s.arrays()
    rays = []
    for i in np.nonzero((t == CAPSULE) | (t == CONVEX))[0][:120]:
        m = 4000
        q, c = pos[i, :4].astype(np.float64), pos[i, 4:7].astype(np.float64)
        u = np.stack([q[:3]] * m)
        w = q[3]

        def rot(v):  # world <- local
            tt = 2 * np.cross(u, v)
            return v + w * tt + np.cross(u, tt)
        if t[i] == CAPSULE:
            h, r = float(prm[i, 0]), float(prm[i, 1])
            phi = rng.uniform(0, 2 * np.pi, m)
            radial_l = np.stack([np.cos(phi), np.zeros(m), np.sin(phi)], 1)
            y = rng.uniform(-h, h, m)
            base_l = np.stack([np.zeros(m), y, np.zeros(m)], 1)
            offset = r * (1.0 + rng.uniform(-0.01, 0.05, m))
            along = rot(np.tile([0.0, 1.0, 0.0], (m, 1)))
        else:
            first, count = int(prm[i].view(np.uint32)[0]), int(prm[i].view(np.uint32)[1])
            v = pool[first:first + count].astype(np.float64)
            radial_l = rng.normal(size=(m, 3))
            radial_l /= np.linalg.norm(radial_l, axis=1, keepdims=True)
            supp = np.max(radial_l @ v.T, axis=1)  # support distance along each radial direction
            ext = np.max(np.abs(v))
            base_l = np.zeros((m, 3))
            offset = supp + ext * rng.uniform(-0.01, 0.05, m)
            along = rot(np.cross(radial_l, rng.normal(size=(m, 3))))
            along /= np.linalg.norm(along, axis=1, keepdims=True)
        radial = rot(radial_l)
        centre = rot(base_l) + c
        rays.append(_grazing_rays(rng, m, centre, radial, along, offset, rng.uniform(1, 60, m)))
    rays = np.concatenate(rays)
    comp = pg.Compound(gpu_ctx, s)
    p, tt, n = comp.cast_rays_and_get_normal(rays, 100.0, solid=solid)
    po, to, no = oracle_lib.Compound(s).cast_rays_and_get_normal(rays, 100.0, solid=solid)
    np.testing.assert_array_equal(p, po)
    hit = po != pg.NO_HIT
    np.testing.assert_array_equal(tt[hit], to[hit])
    np.testing.assert_array_equal(n[hit], no[hit])
    assert 0.1 < hit.mean() < 0.95
