"""Seeded synthetic inputs for the query-path workloads (host-side, numpy).

Random numbers come from a counter-based SplitMix64 (value i of stream s = mix(seed + s*C + (i+1)*G)),
so every array is a pure function of (seed, stream, index) and identical on x86-64 and aarch64.
Workloads:
  - terrain ray casts: a (nx+1) x (nz+1) height-field TriMesh (x, z spacing 1, heights U[0, 4)),
    2 triangles per cell wound counter-clockwise seen from +y, and rays with origins
    U([0, nx) x [10, 20) x [0, nz)) and directions uniform on the downward unit hemisphere.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_STREAM = np.uint64(0xD1B54A32D192ED03)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, stream: int, n: int) -> np.ndarray:
    idx = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + np.uint64(stream) * _STREAM + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, stream: int, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """float64 values in [lo, hi) with 53-bit resolution."""
    u = (splitmix64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def terrain_mesh(nx: int = 256, nz: int = 128, seed: int = 0x9A77E0) -> tuple[np.ndarray, np.ndarray]:
    """Height-field TriMesh: ((nx+1)*(nz+1), 3) f32 vertices and (2*nx*nz, 3) u32 indices."""
    ix, iz = np.meshgrid(np.arange(nx + 1), np.arange(nz + 1), indexing="ij")
    h = uniform(seed, 1, (nx + 1) * (nz + 1), 0.0, 4.0).reshape(nx + 1, nz + 1)
    verts = np.stack([ix.astype(np.float64), h, iz.astype(np.float64)], axis=-1).reshape(-1, 3).astype(np.float32)
    cx, cz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    cx = cx.reshape(-1).astype(np.int64)
    cz = cz.reshape(-1).astype(np.int64)
    v00 = cx * (nz + 1) + cz
    v10 = (cx + 1) * (nz + 1) + cz
    v01 = cx * (nz + 1) + cz + 1
    v11 = (cx + 1) * (nz + 1) + cz + 1
    t0 = np.stack([v00, v01, v10], axis=-1)
    t1 = np.stack([v10, v01, v11], axis=-1)
    idx = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.uint32)
    return verts, idx


def terrain_rays(n: int, nx: int = 256, nz: int = 128, seed: int = 0x9A77E0) -> np.ndarray:
    """(n, 6) f32 rays: origin U([0,nx) x [10,20) x [0,nz)), direction on the downward hemisphere."""
    ox = uniform(seed, 2, n, 0.0, float(nx))
    oy = uniform(seed, 3, n, 10.0, 20.0)
    oz = uniform(seed, 4, n, 0.0, float(nz))
    dy = -uniform(seed, 5, n)
    phi = uniform(seed, 6, n, 0.0, 2.0 * np.pi)
    r = np.sqrt(np.maximum(0.0, 1.0 - dy * dy))
    rays = np.stack([ox, oy, oz, r * np.cos(phi), dy, r * np.sin(phi)], axis=-1)
    return rays.astype(np.float32)


def _log_uniform(seed: int, stream: int, n: int, lo: float, hi: float) -> np.ndarray:
    return np.exp(uniform(seed, stream, n, np.log(lo), np.log(hi)))


def _unit_quats(seed: int, stream: int, n: int) -> np.ndarray:
    """Uniform random unit quaternions (i, j, k, w) by Shoemake's subgroup method, float64."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 1, n, 0.0, 2.0 * np.pi)
    u3 = uniform(seed, stream + 2, n, 0.0, 2.0 * np.pi)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(u2), a * np.cos(u2), b * np.sin(u3), b * np.cos(u3)], axis=-1)
    return q / np.linalg.norm(q, axis=-1, keepdims=True)


def _sphere_dirs(seed: int, stream: int, n: int) -> np.ndarray:
    z = uniform(seed, stream, n, -1.0, 1.0)
    phi = uniform(seed, stream + 1, n, 0.0, 2.0 * np.pi)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=-1)


def ellipsoid_hulls(n_hulls: int, seed: int, stream: int, nmin: int = 8, nmax: int = 256):
    """Vertex clouds of `n_hulls` hulls: N ~ round(log-uniform[nmin, nmax]) points uniform on the unit
    sphere, scaled per axis by U[0.5, 2]. Points on an ellipsoid are all extreme points, so the
    cloud is the hull's vertex set. Returns (pool (sum N, 3) f32, first (n,), count (n,))."""
    counts = np.rint(_log_uniform(seed, stream, n_hulls, nmin, nmax)).astype(np.int64)
    counts = np.clip(counts, nmin, nmax)
    first = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    total = int(counts.sum())
    dirs = _sphere_dirs(seed, stream + 1, total)
    scale = uniform(seed, stream + 3, 3 * n_hulls, 0.5, 2.0).reshape(n_hulls, 3)
    owner = np.repeat(np.arange(n_hulls), counts)
    pool = (dirs * scale[owner]).astype(np.float32)
    return pool, first.astype(np.uint32), counts.astype(np.uint32)


def hull_pairs(n_pairs: int, seed: int = 0x9A77E2, nmin: int = 8, nmax: int = 256):
    """Batched uneven GJK/EPA workload: pair k = (hull 2k at the identity, hull 2k+1 at a random
    relative pose: uniform rotation, translation = unit direction x U[0.5, 3]).
    Returns (ShapeSet, pairs (n, 2) u32)."""
    from .shapes import ShapeSet, CONVEX
    n = 2 * n_pairs
    pool, first, count = ellipsoid_hulls(n, seed, 10, nmin, nmax)
    types = np.full(n, CONVEX, np.uint32)
    params = np.zeros((n, 4), np.float32)
    pu = params.view(np.uint32)
    pu[:, 0] = first
    pu[:, 1] = count
    poses = np.zeros((n, 7), np.float64)
    poses[:, 3] = 1.0
    q = _unit_quats(seed, 20, n_pairs)
    t = _sphere_dirs(seed, 30, n_pairs) * uniform(seed, 32, n_pairs, 0.5, 3.0)[:, None]
    poses[1::2, 0:4] = q
    poses[1::2, 4:7] = t
    pairs = np.stack([np.arange(0, n, 2), np.arange(1, n, 2)], axis=1).astype(np.uint32)
    return ShapeSet.from_arrays(types, params, poses.astype(np.float32), pool), pairs


def mixed_contact_pairs(n_pairs: int, seed: int = 0x9A77E5, nmin: int = 8, nmax: int = 256):
    """The uneven GJK/EPA workload with primitives mixed in: each shape of pair k (shapes 2k at the
    identity and 2k+1 at a random relative pose, as hull_pairs) is, uniformly, a ball (radius
    log-uniform [0.5, 2]), a cuboid (half extents log-uniform [0.5, 2]), a capsule (half height and
    radius log-uniform [0.25, 1.5]) or a hull of N ~ log-uniform[nmin, nmax] points on an ellipsoid.
    Returns (ShapeSet, pairs (n, 2) u32)."""
    from .shapes import ShapeSet, BALL, CUBOID, CAPSULE, CONVEX
    n = 2 * n_pairs
    kinds = (splitmix64(seed, 1, n) % np.uint64(4)).astype(np.uint32)
    types = np.array([BALL, CUBOID, CAPSULE, CONVEX], np.uint32)[kinds]
    params = np.zeros((n, 4), np.float32)
    pu = params.view(np.uint32)
    ball, cub, cap, cvx = types == BALL, types == CUBOID, types == CAPSULE, types == CONVEX
    params[ball, 0] = _log_uniform(seed, 2, n, 0.5, 2.0)[ball]
    for j in range(3):
        params[cub, j] = _log_uniform(seed, 3 + j, n, 0.5, 2.0)[cub]
    params[cap, 0] = _log_uniform(seed, 6, n, 0.25, 1.5)[cap]
    params[cap, 1] = _log_uniform(seed, 7, n, 0.25, 1.5)[cap]
    hull_ids = np.nonzero(cvx)[0]
    pool, first, count = ellipsoid_hulls(len(hull_ids), seed, 10, nmin, nmax)
    pu[hull_ids, 0] = first
    pu[hull_ids, 1] = count
    poses = np.zeros((n, 7), np.float64)
    poses[:, 3] = 1.0
    poses[1::2, 0:4] = _unit_quats(seed, 20, n_pairs)
    poses[1::2, 4:7] = _sphere_dirs(seed, 30, n_pairs) * uniform(seed, 32, n_pairs, 0.5, 3.0)[:, None]
    pairs = np.stack([np.arange(0, n, 2), np.arange(1, n, 2)], axis=1).astype(np.uint32)
    return ShapeSet.from_arrays(types, params, poses.astype(np.float32), pool), pairs


def shape_cast_pairs(n_pairs: int, seed: int = 0x9A77E6, spread: float = 6.0):
    """Shape-casting workload: the mixed_contact_pairs shapes with the second shape of each pair moved
    `spread` away in a random direction; per-shape velocities N(0, 0.3^2) per axis, plus, for the
    second shape, a speed U[0.5, 2] back towards the first. Returns (ShapeSet, pairs (n, 2) u32,
    velocities (2n, 3) f32)."""
    from .shapes import ShapeSet
    s, pairs = mixed_contact_pairs(n_pairs, seed=seed)
    t, prm, pos, pool = s.arrays()
    pos = pos.copy()
    d = _sphere_dirs(seed, 40, n_pairs).astype(np.float32)
    pos[1::2, 4:7] += spread * d
    vels = np.stack([uniform(seed, 43 + j, 2 * n_pairs, -0.5, 0.5) for j in range(3)], axis=1).astype(np.float32)
    vels[1::2] -= d * uniform(seed, 46, n_pairs, 0.5, 2.0)[:, None].astype(np.float32)
    return ShapeSet.from_arrays(t, prm, pos, pool), pairs, vels


def broadphase_shapes(n: int = 131072, extent: float = 200.0, seed: int = 0x9A77E1):
    """Broadphase workload: n shapes, even indices balls (radius log-uniform [0.25, 4]), odd indices
    cuboids (half extents log-uniform [0.25, 4], uniform rotation), centres U([-extent, extent)^3)."""
    from .shapes import ShapeSet, BALL, CUBOID
    types = np.where(np.arange(n) % 2 == 0, BALL, CUBOID).astype(np.uint32)
    params = np.zeros((n, 4), np.float64)
    params[:, 0] = _log_uniform(seed, 1, n, 0.25, 4.0)
    params[:, 1] = _log_uniform(seed, 2, n, 0.25, 4.0)
    params[:, 2] = _log_uniform(seed, 3, n, 0.25, 4.0)
    params[types == BALL, 1:] = 0.0
    poses = np.zeros((n, 7), np.float64)
    poses[:, 3] = 1.0
    q = _unit_quats(seed, 4, n)
    cub = types == CUBOID
    poses[cub, 0:4] = q[cub]
    poses[:, 4] = uniform(seed, 8, n, -extent, extent)
    poses[:, 5] = uniform(seed, 9, n, -extent, extent)
    poses[:, 6] = uniform(seed, 10, n, -extent, extent)
    return ShapeSet.from_arrays(types, params.astype(np.float32), poses.astype(np.float32))


def primitive_pairs(n_pairs: int, seed: int = 0x9A77E3, hulls: bool = True, n_hull_shapes: int = 4096):
    """Contact-manifold workload: pair k = (shape 2k at the identity, shape 2k+1 at a random relative
    pose: uniform rotation, translation = unit direction x U[0.5, 3]). Kinds are drawn uniformly per
    shape among balls (radius U[0.5, 1]), cuboids (half extents U[0.4, 1]), capsules (half height
    U[0.2, 0.8], radius U[0.3, 0.6]) and, with `hulls`, convex hulls of 16-64 points on spheres
    scaled per axis by U[0.25, 1] (ConvexPolyhedron topology; `n_hull_shapes` distinct hulls shared
    by all hull shapes). Returns (types u32, params f32 (n, 4), poses f32 (n, 7), pool, polyhedra,
    pairs (n_pairs, 2) u32); polyhedra is None without hulls."""
    from .shapes import BALL, CUBOID, CAPSULE, CONVEX
    n = 2 * n_pairs
    kinds = 4 if hulls else 3
    types = (splitmix64(seed, 1, n) % np.uint64(kinds)).astype(np.uint32)
    params = np.zeros((n, 4), np.float64)
    ball, cub, cap = types == BALL, types == CUBOID, types == CAPSULE
    params[ball, 0] = uniform(seed, 2, n, 0.5, 1.0)[ball]
    for j in range(3):
        params[cub, j] = uniform(seed, 3 + j, n, 0.4, 1.0)[cub]
    params[cap, 0] = uniform(seed, 6, n, 0.2, 0.8)[cap]
    params[cap, 1] = uniform(seed, 7, n, 0.3, 0.6)[cap]
    params = params.astype(np.float32)
    pool = np.zeros((0, 3), np.float32)
    poly = None
    if hulls:
        from .polyhedra import build_polyhedra
        cloud, first, count = ellipsoid_hulls(n_hull_shapes, seed, 50, 16, 64)
        # ellipsoid_hulls scales by U[0.5, 2]; halve to keep sizes comparable with the primitives
        pool, hull_rec, topo = build_polyhedra(cloud * 0.5, first, count)
        poly = (hull_rec, topo)
        cvx = types == CONVEX
        pick = (splitmix64(seed, 8, n) % np.uint64(n_hull_shapes)).astype(np.int64)
        pu = params.view(np.uint32)
        pu[cvx, 0] = hull_rec[pick[cvx], 0]
        pu[cvx, 1] = hull_rec[pick[cvx], 1]
        pu[cvx, 2] = np.where(hull_rec[pick[cvx], 6] == 1, pick[cvx] + 1, 0).astype(np.uint32)
    poses = np.zeros((n, 7), np.float64)
    poses[:, 3] = 1.0
    poses[1::2, 0:4] = _unit_quats(seed, 20, n_pairs)
    poses[1::2, 4:7] = _sphere_dirs(seed, 30, n_pairs) * uniform(seed, 32, n_pairs, 0.5, 3.0)[:, None]
    pairs = np.stack([np.arange(0, n, 2), np.arange(1, n, 2)], axis=1).astype(np.uint32)
    return types, params, poses.astype(np.float32), pool, poly, pairs


def drifted_poses(poses: np.ndarray, frame: int, seed: int = 0x9A77E4, dt: float = 1.0 / 60.0, speed: float = 0.3,
                  spin: float = 0.5) -> np.ndarray:
    """Poses after `frame` steps of dt: each shape moves with a velocity U([-speed, speed]^3) and
    spins with an angular velocity U([-spin, spin]^3) (exponential map, renormalised)."""
    n = len(poses)
    v = np.stack([uniform(seed, 40 + j, n, -speed, speed) for j in range(3)], axis=1)
    w = np.stack([uniform(seed, 43 + j, n, -spin, spin) for j in range(3)], axis=1)
    out = poses.astype(np.float64).copy()
    out[:, 4:7] += v * (dt * frame)
    ang = w * (dt * frame)
    th = np.linalg.norm(ang, axis=1)
    ax = ang / np.maximum(th, 1e-30)[:, None]
    s, c = np.sin(th / 2), np.cos(th / 2)
    di, dj, dk, dw = ax[:, 0] * s, ax[:, 1] * s, ax[:, 2] * s, c
    qi, qj, qk, qw = out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy(), out[:, 3].copy()
    out[:, 0] = dw * qi + di * qw + dj * qk - dk * qj
    out[:, 1] = dw * qj - di * qk + dj * qw + dk * qi
    out[:, 2] = dw * qk + di * qj - dj * qi + dk * qw
    out[:, 3] = dw * qw - di * qi - dj * qj - dk * qk
    out[:, :4] /= np.linalg.norm(out[:, :4], axis=1, keepdims=True)
    return out.astype(np.float32)


def frame_scene(n: int = 262144, n_rays: int = 4194304, extent: float = 400.0, seed: int = 0x9A77E4):
    """Per-frame pipeline workload: n shapes, kinds drawn uniformly per shape among balls (radius
    log-uniform [0.25, 4]), cuboids (half extents log-uniform [0.25, 4], uniform rotation), capsules
    (half height and radius log-uniform [0.25, 4]) and convex hulls of 16-64 points on spheres scaled
    per axis by U[0.5, 2] (ConvexPolyhedron topology, one hull per hull shape); centres
    U([-extent, extent)^3), velocities U[-5, 5]^3, angular velocities U[-1, 1]^3. Rays: origins
    U([-extent, extent)^3), directions uniform on the sphere.
    Returns (types, params, poses, pool, polyhedra, velocities (n, 6), rays (n_rays, 6))."""
    from .shapes import BALL, CUBOID, CAPSULE, CONVEX
    from .polyhedra import build_polyhedra
    types = (splitmix64(seed, 1, n) % np.uint64(4)).astype(np.uint32)
    params = np.zeros((n, 4), np.float64)
    ball, cub, cap, cvx = types == BALL, types == CUBOID, types == CAPSULE, types == CONVEX
    params[ball, 0] = _log_uniform(seed, 2, n, 0.25, 4.0)[ball]
    for j in range(3):
        params[cub, j] = _log_uniform(seed, 3 + j, n, 0.25, 4.0)[cub]
    params[cap, 0] = _log_uniform(seed, 6, n, 0.25, 4.0)[cap]
    params[cap, 1] = _log_uniform(seed, 7, n, 0.25, 4.0)[cap]
    params = params.astype(np.float32)
    hull_ids = np.nonzero(cvx)[0]
    cloud, first, count = ellipsoid_hulls(len(hull_ids), seed, 50, 16, 64)
    pool, hulls, topo = build_polyhedra(cloud, first, count)
    pu = params.view(np.uint32)
    pu[hull_ids, 0] = hulls[:, 0]
    pu[hull_ids, 1] = hulls[:, 1]
    pu[hull_ids, 2] = np.where(hulls[:, 6] == 1, np.arange(len(hull_ids)) + 1, 0).astype(np.uint32)
    poses = np.zeros((n, 7), np.float64)
    poses[:, 0:4] = _unit_quats(seed, 20, n)
    for j in range(3):
        poses[:, 4 + j] = uniform(seed, 30 + j, n, -extent, extent)
    vel = np.zeros((n, 6), np.float64)
    for j in range(3):
        vel[:, j] = uniform(seed, 40 + j, n, -5.0, 5.0)
        vel[:, 3 + j] = uniform(seed, 43 + j, n, -1.0, 1.0)
    rays = np.zeros((n_rays, 6), np.float64)
    for j in range(3):
        rays[:, j] = uniform(seed, 60 + j, n_rays, -extent, extent)
    rays[:, 3:] = _sphere_dirs(seed, 63, n_rays)
    return (types, params, poses.astype(np.float32), pool, (hulls, topo), vel.astype(np.float32), rays.astype(np.float32))
