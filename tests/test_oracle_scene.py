"""The oracle's frame loop (CPU): integration rule D-5 and pipeline invariants."""
import numpy as np

from tests._contact_cases import hull_scene
from tests._helpers import brute_force_pairs


def test_integrate_rule(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(0)
    q = rng.normal(size=(500, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    poses = np.concatenate([q, rng.uniform(-10, 10, (500, 3))], axis=1).astype(np.float32)
    vel = np.concatenate([rng.uniform(-5, 5, (500, 3)), rng.uniform(-1, 1, (500, 3))], axis=1).astype(np.float32)
    dt = np.float32(1.0 / 60.0)
    out = O.integrate(poses, vel, float(dt))
    np.testing.assert_array_equal(out[:, 4:], poses[:, 4:] + vel[:, :3] * dt)
    np.testing.assert_allclose(np.linalg.norm(out[:, :4].astype(np.float64), axis=1), 1.0, atol=1e-6)
    # first-order rotation: the relative rotation angle is |w| dt to first order
    qa, qb = poses[:, :4].astype(np.float64), out[:, :4].astype(np.float64)
    cos_half = np.abs(np.sum(qa * qb, axis=1))
    ang = 2 * np.arccos(np.clip(cos_half, -1, 1))
    np.testing.assert_allclose(ang, np.linalg.norm(vel[:, 3:], axis=1) * dt, rtol=1e-2, atol=2e-4)
    # zero angular velocity keeps the rotation up to renormalisation
    vel0 = vel.copy()
    vel0[:, 3:] = 0
    np.testing.assert_allclose(O.integrate(poses, vel0, float(dt))[:, :4], poses[:, :4], atol=1e-7)


def test_scene_frames_invariants(oracle_lib):
    O = oracle_lib
    s, _ = hull_scene(300, 12, extent=5.0)
    rng = np.random.default_rng(2)
    vel = np.concatenate([rng.uniform(-5, 5, (300, 3)), rng.uniform(-1, 1, (300, 3))], axis=1).astype(np.float32)
    a = O.scene_frames(s, vel, 0.1, 1.0 / 60.0, 3)
    b = O.scene_frames(s, vel, 0.1, 1.0 / 60.0, 3, threads=1)
    np.testing.assert_array_equal(a["poses"], b["poses"])
    np.testing.assert_array_equal(a["pairs"], b["pairs"])
    np.testing.assert_array_equal(a["manifolds"], b["manifolds"])
    # the pair set is every pair of overlapping loosened AABBs of the final poses
    aabbs = O.shape_aabbs(s.with_poses(a["poses"]), 0.05)
    np.testing.assert_array_equal(a["pairs"], brute_force_pairs(aabbs))
    assert np.all(a["manifolds"][:, 1] == 0)
