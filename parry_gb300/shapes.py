"""Host-side description of a set of convex shapes in the C-ABI layout (parrygpu_shapes).

Each shape has a type, four parameters and a pose (Isometry as pose7 = qi, qj, qk, qw, tx, ty, tz):

    type      parry3d shape                         params
    BALL      Ball::new(r)                          r, 0, 0, 0
    CUBOID    Cuboid::new(half_extents)             hx, hy, hz, 0
    CAPSULE   Capsule::new_y(half_height, radius)   half_height, radius, 0, 0
    CONVEX    ConvexPolyhedron (vertex cloud)       first vertex, vertex count (u32 bits), 0, 0
    TRIANGLE  Triangle::new(a, b, c)                first vertex (u32 bits), 3, 0, 0

Convex and triangle vertices live in one shared pool (n_vertices x 3 floats).
"""
from __future__ import annotations

import numpy as np

BALL, CUBOID, CAPSULE, CONVEX, TRIANGLE = 0, 1, 2, 3, 4
IDENTITY_POSE = (0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0)


def pose7(translation=(0.0, 0.0, 0.0), quat=(0.0, 0.0, 0.0, 1.0)) -> tuple:
    return (float(quat[0]), float(quat[1]), float(quat[2]), float(quat[3]),
            float(translation[0]), float(translation[1]), float(translation[2]))


class ShapeSet:
    def __init__(self):
        self._types: list[int] = []
        self._params: list[tuple] = []
        self._poses: list[tuple] = []
        self._pool: list[np.ndarray] = []
        self._pool_len = 0
        self._arrays = None

    def __len__(self) -> int:
        return len(self._types) if self._arrays is None else len(self._arrays[0])

    def _add(self, t, params, pose):
        assert self._arrays is None, "ShapeSet built from arrays is immutable"
        self._types.append(t)
        self._params.append(params)
        self._poses.append(tuple(pose) if pose is not None else IDENTITY_POSE)
        return len(self._types) - 1

    def add_ball(self, radius, pose=None):
        return self._add(BALL, (radius, 0.0, 0.0, 0.0), pose)

    def add_cuboid(self, half_extents, pose=None):
        return self._add(CUBOID, (half_extents[0], half_extents[1], half_extents[2], 0.0), pose)

    def add_capsule(self, half_height, radius, pose=None):
        return self._add(CAPSULE, (half_height, radius, 0.0, 0.0), pose)

    def _add_points(self, t, pts, pose):
        pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
        first = self._pool_len
        self._pool.append(pts)
        self._pool_len += len(pts)
        return self._add(t, ("u32", first, len(pts)), pose), (first, len(pts))

    def add_convex(self, points, pose=None):
        return self._add_points(CONVEX, points, pose)[0]

    def add_triangle(self, a, b, c, pose=None):
        return self._add_points(TRIANGLE, [a, b, c], pose)[0]

    @classmethod
    def from_arrays(cls, types, params, poses, pool=None) -> "ShapeSet":
        s = cls()
        pool = np.zeros((0, 3), np.float32) if pool is None else np.ascontiguousarray(pool, np.float32).reshape(-1, 3)
        s._arrays = (np.ascontiguousarray(types, np.uint32), np.ascontiguousarray(params, np.float32).reshape(-1, 4),
                     np.ascontiguousarray(poses, np.float32).reshape(-1, 7), pool)
        return s

    def arrays(self):
        """(types u32 (n,), params f32 (n, 4), poses f32 (n, 7), pool f32 (m, 3))."""
        if self._arrays is not None:
            return self._arrays
        types = np.array(self._types, dtype=np.uint32)
        params = np.zeros((len(self._types), 4), dtype=np.float32)
        pu = params.view(np.uint32)
        for i, (t, p) in enumerate(zip(self._types, self._params)):
            if t in (CONVEX, TRIANGLE):
                pu[i, 0], pu[i, 1] = p[1], p[2]  # first vertex, count as u32 bit patterns
            else:
                params[i] = p
        poses = np.array(self._poses, dtype=np.float32).reshape(-1, 7)
        pool = np.concatenate(self._pool).astype(np.float32) if self._pool else np.zeros((0, 3), np.float32)
        return types, params, poses, pool
