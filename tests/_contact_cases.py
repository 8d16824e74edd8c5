"""Builds the reference's known-answer contact cases as ShapeSets + pair lists (shared by the
oracle tests and the GPU parity tests)."""
import json
from pathlib import Path

import numpy as np

from parry_gb300.shapes import ShapeSet, pose7

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def cuboid_epa():
    c = KA["cuboid_cuboid_epa"]
    s = ShapeSet()
    pairs = []
    for case in c["cases"]:
        a = s.add_cuboid(c["half_extents"], pose7(case["pos1"]))
        b = s.add_cuboid(c["half_extents"], pose7(case["pos2"]))
        pairs.append((a, b))
    return s, np.array(pairs, np.uint32), c


def triangle_touch():
    c = KA["triangle_vertex_touches_triangle_edge_epa"]
    s = ShapeSet()
    a = s.add_triangle(*c["tri1"])
    b = s.add_triangle(*c["tri2"])
    return s, np.array([(a, b)], np.uint32), c


def ball_ball():
    c = KA["ball_ball_prediction"]
    s = ShapeSet()
    a = s.add_ball(c["radius"], pose7(c["pos1"]))
    b = s.add_ball(c["radius"], pose7(c["pos2"]))
    return s, np.array([(a, b)], np.uint32), c


def ball_cuboid():
    c = KA["ball_cuboid_contact_query"]
    s = ShapeSet()
    cub = s.add_cuboid(c["cuboid_half_extents"])
    pairs = []
    for case in c["cases"]:
        b = s.add_ball(c["ball_radius"], pose7(case["ball_pos"]))
        pairs.append((b, cub))
    return s, np.array(pairs, np.uint32), c


def cuboid_ray():
    c = KA["cuboid_ray_doc_test"]
    s = ShapeSet()
    s.add_cuboid(c["half_extents"])
    return s, np.array([c["ray"]], np.float32), c


def solid_ray_cast():
    c = KA["solid_ray_cast3d"]
    s = ShapeSet()
    s.add_cuboid(c["half_extents"])
    return s, c


def mixed_scene(n: int, seed: int, extent: float = 6.0):
    """Balls, cuboids, capsules, convex hulls and triangles at random poses in a cube."""
    from parry_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    s = ShapeSet()
    pool, first, count = W.ellipsoid_hulls(32, seed=seed, stream=1, nmin=8, nmax=64)
    for i in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pose = pose7(rng.uniform(-extent, extent, 3), q)
        t = i % 5
        if t == 0:
            s.add_ball(rng.uniform(0.3, 1.5), pose)
        elif t == 1:
            s.add_cuboid(rng.uniform(0.3, 1.5, 3), pose)
        elif t == 2:
            s.add_capsule(rng.uniform(0.2, 1.2), rng.uniform(0.2, 0.8), pose)
        elif t == 3:
            h = i % 32
            s.add_convex(pool[first[h]:first[h] + count[h]], pose)
        else:
            s.add_triangle(*rng.uniform(-1.2, 1.2, (3, 3)), pose)
    return s


def primitive_scene(n: int, seed: int, extent: float = 4.0):
    """(types, params, poses) of balls, cuboids and capsules (types cycling 0, 1, 2) at random poses:
    the shape kinds with contact-manifold generators."""
    rng = np.random.default_rng(seed)
    types = (np.arange(n) % 3).astype(np.uint32)
    params = np.zeros((n, 4), np.float32)
    for i in range(n):
        if types[i] == 0:
            params[i, 0] = rng.uniform(0.3, 1.5)
        elif types[i] == 1:
            params[i, :3] = rng.uniform(0.3, 1.5, 3)
        else:
            params[i, :2] = (rng.uniform(0.2, 1.2), rng.uniform(0.2, 0.8))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    poses = np.concatenate([q, rng.uniform(-extent, extent, (n, 3))], axis=1).astype(np.float32)
    return types, params, poses


def moved_poses(poses: np.ndarray, frame: int, seed: int, step: float = 0.01, angle: float = 0.01) -> np.ndarray:
    """Poses after `frame` steps of a small per-shape drift and spin (renormalised quaternions)."""
    rng = np.random.default_rng(seed)
    n = len(poses)
    v = rng.normal(size=(n, 3)) * step
    w = rng.normal(size=(n, 3)) * angle
    out = poses.astype(np.float64).copy()
    out[:, 4:7] += v * frame
    # q <- exp(w * frame / 2) * q
    th = np.linalg.norm(w, axis=1) * frame
    ax = w / np.maximum(np.linalg.norm(w, axis=1, keepdims=True), 1e-30)
    dq = np.concatenate([ax * np.sin(th / 2)[:, None], np.cos(th / 2)[:, None]], axis=1)
    qi, qj, qk, qw = out[:, 0], out[:, 1], out[:, 2], out[:, 3]
    di, dj, dk, dw = dq[:, 0], dq[:, 1], dq[:, 2], dq[:, 3]
    out[:, 0] = dw * qi + di * qw + dj * qk - dk * qj
    out[:, 1] = dw * qj - di * qk + dj * qw + dk * qi
    out[:, 2] = dw * qk + di * qj - dj * qi + dk * qw
    out[:, 3] = dw * qw - di * qi - dj * qj - dk * qk
    out[:, :4] /= np.linalg.norm(out[:, :4], axis=1, keepdims=True)
    return out.astype(np.float32)


def hull_scene(n: int, seed: int, extent: float = 5.0):
    """Balls, cuboids, capsules and convex hulls (16-64 points on scaled spheres, built as
    ConvexPolyhedron topology), types cycling 0..3, at random poses. Returns (ShapeSet, poses)."""
    from parry_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    s = ShapeSet()
    pool, first, count = W.ellipsoid_hulls(64, seed=seed, stream=3, nmin=16, nmax=64)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    poses = np.concatenate([q, rng.uniform(-extent, extent, (n, 3))], axis=1).astype(np.float32)
    for i in range(n):
        t = i % 4
        if t == 0:
            s.add_ball(rng.uniform(0.3, 1.2), poses[i])
        elif t == 1:
            s.add_cuboid(rng.uniform(0.3, 1.2, 3), poses[i])
        elif t == 2:
            s.add_capsule(rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.6), poses[i])
        else:
            h = (i // 4) % 64
            s.add_convex_hull(pool[first[h]:first[h] + count[h]], poses[i])
    return s, poses


def toi_cases():
    """The reference's time-of-impact tests as (ShapeSet, pairs (k, 2), per-shape velocities (n, 3),
    expectations): each expectation is ("toi", value), ("toi_rel", value), ("none",) or ("some",)."""
    s = ShapeSet()
    pairs, vels, expect = [], [], []

    def add(shape_a, shape_b, va, vb, e):
        pairs.append((shape_a, shape_b))
        vels.extend([va, vb])
        expect.append(e)

    c = KA["toi_ball_ball"]
    a = s.add_ball(c["radius"], pose7([0, 0, 0]))
    b = s.add_ball(c["radius"], pose7(c["pos2"]))
    add(a, b, c["vel1"], c["vel2"], ("toi", c["expect_toi"]))
    c = KA["toi_ball_triangle_tiny_velocity"]
    a = s.add_ball(c["radius"], pose7([0, 0, 0]))
    b = s.add_triangle(*c["triangle"], pose=pose7(c["pos2"]))
    add(a, b, c["vel1"], c["vel2"], ("none",))
    c = KA["toi_ball_cuboid"]
    for case in c["cases"]:
        a = s.add_ball(c["ball_radius"], pose7(case["ball_pos"]))
        b = s.add_cuboid(c["cuboid_half_extents"], pose7([0, 0, 0]))
        if "expect_toi" in case:
            e = ("toi", case["expect_toi"])
        elif "expect_toi_relative_eq" in case:
            dv = np.array(case["ball_vel"]) - np.array(case["cuboid_vel"])
            e = ("toi_rel", (np.sqrt(3.0) - 1.0) / np.linalg.norm(dv))
        else:
            e = ("none",)
        add(a, b, case["ball_vel"], case["cuboid_vel"], e)
    c = KA["toi_still_cuboids"]
    for case in c["cases"]:
        a = s.add_cuboid(c["half_extents"], pose7(c["pos1"]))
        b = s.add_cuboid(c["half_extents"], pose7([0, 0, 0]))
        add(a, b, [0.0, case["v_y"], 0.0], [0.0, 0.0, 0.0], ("none",) if case["expect"] is None else ("some",))
    return s, np.array(pairs, np.uint32), np.array(vels, np.float32), expect


def check_toi(status, out, expect):
    for k, e in enumerate(expect):
        if e[0] == "none":
            assert status[k] == 255, (k, e, status[k])
        else:
            assert status[k] != 255, (k, e)
            if e[0] == "toi":
                assert out[k, 0] == np.float32(e[1]), (k, out[k, 0], e)
            elif e[0] == "toi_rel":
                assert abs(out[k, 0] - e[1]) <= 1e-5 * abs(e[1]), (k, out[k, 0], e)
