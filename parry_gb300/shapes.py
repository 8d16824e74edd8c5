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
        self._pts: list = []          # per shape: vertex array (convex / triangle) or None
        self._hull: list[bool] = []   # per shape: build ConvexPolyhedron topology for it
        self._arrays = None
        self._poly = None

    def __len__(self) -> int:
        return len(self._types) if self._arrays is None else len(self._arrays[0])

    def _add(self, t, params, pose, pts=None, hull=False):
        assert self._arrays is None, "ShapeSet built from arrays is immutable"
        self._types.append(t)
        self._params.append(params)
        self._poses.append(tuple(pose) if pose is not None else IDENTITY_POSE)
        self._pts.append(None if pts is None else np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3))
        self._hull.append(hull)
        self._built = None
        return len(self._types) - 1

    def add_ball(self, radius, pose=None):
        return self._add(BALL, (radius, 0.0, 0.0, 0.0), pose)

    def add_cuboid(self, half_extents, pose=None):
        return self._add(CUBOID, (half_extents[0], half_extents[1], half_extents[2], 0.0), pose)

    def add_capsule(self, half_height, radius, pose=None):
        return self._add(CAPSULE, (half_height, radius, 0.0, 0.0), pose)

    def add_convex(self, points, pose=None):
        """A convex shape given by its vertex cloud (support-map queries; no manifold topology)."""
        return self._add(CONVEX, None, pose, points)

    def add_convex_hull(self, points, pose=None):
        """ConvexPolyhedron::from_convex_hull(points): the hull's vertices plus its face topology."""
        return self._add(CONVEX, None, pose, points, hull=True)

    def add_triangle(self, a, b, c, pose=None):
        return self._add(TRIANGLE, None, pose, [a, b, c])

    @classmethod
    def from_arrays(cls, types, params, poses, pool=None, polyhedra=None) -> "ShapeSet":
        """polyhedra: None or (hulls (h, 8) u32, topology dict) as parry_gb300.polyhedra builds them,
        with vertex_ranges parallel to `pool`; convex params[2] (u32 bits) = hull index + 1."""
        s = cls()
        pool = np.zeros((0, 3), np.float32) if pool is None else np.ascontiguousarray(pool, np.float32).reshape(-1, 3)
        s._arrays = (np.ascontiguousarray(types, np.uint32), np.ascontiguousarray(params, np.float32).reshape(-1, 4),
                     np.ascontiguousarray(poses, np.float32).reshape(-1, 7), pool)
        s._poly = polyhedra
        return s

    def with_poses(self, poses) -> "ShapeSet":
        """The same shapes at other poses (shares the other arrays)."""
        t, p, _, pool = self.arrays()
        return ShapeSet.from_arrays(t, p, poses, pool, self.polyhedra())

    def _build(self):
        from .polyhedra import build_polyhedra, empty_topology
        n = len(self._types)
        types = np.array(self._types, dtype=np.uint32)
        params = np.zeros((n, 4), dtype=np.float32)
        pu = params.view(np.uint32)
        hull_ids = [i for i in range(n) if self._hull[i]]
        hull_pts = hulls = topo = None
        if hull_ids:
            clouds = [self._pts[i] for i in hull_ids]
            counts = np.array([len(c) for c in clouds], np.uint32)
            firsts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
            hull_pts, hulls, topo = build_polyhedra(np.concatenate(clouds), firsts, counts)
        pool_parts, vr_parts = [], []
        off = 0
        hk = 0
        for i, (t, prm) in enumerate(zip(self._types, self._params)):
            if self._pts[i] is None:
                params[i] = prm
                continue
            if self._hull[i]:
                r = hulls[hk]
                pts = hull_pts[r[0]:r[0] + r[1]]
                vr_parts.append(topo["vertex_ranges"][r[0]:r[0] + r[1]])
                hulls[hk, 0] = off
                pu[i, 2] = hk + 1 if r[6] else 0
                hk += 1
            else:
                pts = self._pts[i]
                vr_parts.append(np.zeros((len(pts), 2), np.uint32))
            pu[i, 0], pu[i, 1] = off, len(pts)
            pool_parts.append(pts)
            off += len(pts)
        poses = np.array(self._poses, dtype=np.float32).reshape(-1, 7)
        pool = np.concatenate(pool_parts).astype(np.float32) if pool_parts else np.zeros((0, 3), np.float32)
        poly = None
        if hull_ids:
            topo = dict(topo)
            topo["vertex_ranges"] = np.ascontiguousarray(np.concatenate(vr_parts), np.uint32)
            poly = (hulls, topo)
        self._built = ((types, params, poses, pool), poly)

    def arrays(self):
        """(types u32 (n,), params f32 (n, 4), poses f32 (n, 7), pool f32 (m, 3))."""
        if self._arrays is not None:
            return self._arrays
        if getattr(self, "_built", None) is None:
            self._build()
        return self._built[0]

    def polyhedra(self):
        """None, or (hulls (h, 8) u32, topology dict) in the parrygpu_polyhedra layout."""
        if self._arrays is not None:
            return self._poly
        if getattr(self, "_built", None) is None:
            self._build()
        return self._built[1]
