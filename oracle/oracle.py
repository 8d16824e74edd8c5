"""Oracle (test infrastructure only): ctypes wrapper over liboracle.so, the C++ restatement of
parry3d's query path (f32 = parry3d, f64 = parry3d-f64).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this, as
the checker or the timed CPU baseline. The product (parry_gb300, libparrygpu.so) never does.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_lib = None

P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I32 = C.c_int
F32 = C.c_float

_SIGS = {
    "oracle_trimesh_new_f32": (P, [P, U32, P, U32]),
    "oracle_trimesh_new_f64": (P, [P, U32, P, U32]),
    "oracle_trimesh_free_f32": (None, [P]),
    "oracle_trimesh_free_f64": (None, [P]),
    "oracle_trimesh_cast_rays_f32": (None, [P, P, P, U64, F32, I32, I32, P, P, P, P]),
    "oracle_trimesh_cast_rays_f64": (None, [P, P, P, U64, F32, I32, I32, P, P, P, P]),
    "oracle_trimesh_bvh_nodes_f32": (U32, [P, P, U32]),
    "oracle_bvh_new_f32": (P, [P, U32]),
    "oracle_bvh_free_f32": (None, [P]),
    "oracle_bvh_nodes_f32": (U32, [P, P, U32]),
    "oracle_bvh_refit_f32": (None, [P, P, U32]),
    "oracle_bvh_self_pairs_f32": (P, [P]),
    "oracle_bvh_leaf_pairs_f32": (P, [P, P]),
    "oracle_shape_aabbs_f32": (None, [P, P, P, P, U32, U64, F32, P]),
    "oracle_contacts_f32": (None, [P, P, P, P, U32, U64, P, U64, F32, P, I32, P, P, P]),
    "oracle_cast_shapes_f32": (None, [P, P, P, P, U32, U64, P, U64, P, P, I32, P, P, P]),
    "oracle_inv_mul_f32": (None, [P, P, U64, P]),
    "oracle_cast_shapes_f64": (None, [P, P, P, P, U32, U64, P, U64, P, P, I32, P, P, P]),
    "oracle_contacts_f64": (None, [P, P, P, P, U32, U64, P, U64, F32, P, I32, P, P, P]),
    "oracle_compound_new_f32": (P, [P, P, P, P, U32, U64]),
    "oracle_compound_new_f64": (P, [P, P, P, P, U32, U64]),
    "oracle_compound_free_f32": (None, [P]),
    "oracle_compound_free_f64": (None, [P]),
    "oracle_compound_cast_rays_f32": (None, [P, P, P, U64, F32, I32, I32, I32, P, P, P, P]),
    "oracle_compound_cast_rays_f64": (None, [P, P, P, U64, F32, I32, I32, I32, P, P, P, P]),
    "oracle_manifolds_f32": (None, [P, P, P, P, U32, U64, P, P, U64, F32, I32, P, P, P, U64, P]),
    "oracle_trimesh_pseudo_normals_f32": (None, [P, U32, P, U32, P, P]),
    "oracle_project_local_normals_f32": (None, [P, P, U64, P, P]),
    "oracle_integrate_f32": (None, [P, P, U64, F32]),
    "oracle_pairs_count": (U64, [P]),
    "oracle_pairs_copy": (None, [P, P]),
    "oracle_pairs_free": (None, [P]),
}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _HERE / "liboracle.so"
        if not path.exists():
            from . import build as _b  # type: ignore
            _b.build()
        l = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def default_threads() -> int:
    return os.cpu_count() or 1


class TriMesh:
    """Reference TriMesh (binned BVH) with cast_ray_and_get_normal in f32 or f64."""

    def __init__(self, vertices: np.ndarray, indices: np.ndarray, precision: str = "f32"):
        self.v = np.ascontiguousarray(vertices, dtype=np.float32)
        self.i = np.ascontiguousarray(indices, dtype=np.uint32)
        self.prec = precision
        self.n_triangles = self.i.shape[0]
        self._h = getattr(lib(), f"oracle_trimesh_new_{precision}")(_p(self.v), self.v.shape[0], _p(self.i), self.i.shape[0])

    def cast_rays_and_get_normal(self, rays: np.ndarray, max_toi: float, pose: np.ndarray | None = None,
                                 lowest_index: bool = True, threads: int | None = None, want_stats: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        dt = np.float32 if self.prec == "f32" else np.float64
        feat = np.empty(n, dtype=np.uint32)
        toi = np.empty(n, dtype=dt)
        nrm = np.empty((n, 3), dtype=dt)
        stats = np.zeros(2, dtype=np.uint64)
        pz = None if pose is None else np.ascontiguousarray(pose, dtype=np.float32)
        getattr(lib(), f"oracle_trimesh_cast_rays_{self.prec}")(
            self._h, _p(pz), _p(rays), n, float(max_toi), 1 if lowest_index else 0,
            threads if threads is not None else default_threads(), _p(feat), _p(toi), _p(nrm),
            _p(stats) if want_stats else None)
        if want_stats:
            return feat, toi, nrm, {"wide_visits": int(stats[0]), "leaf_tests": int(stats[1])}
        return feat, toi, nrm

    def bvh_nodes(self) -> np.ndarray:
        n = lib().oracle_trimesh_bvh_nodes_f32(self._h, None, 0)
        raw = np.empty(n * 16, dtype=np.float32)
        lib().oracle_trimesh_bvh_nodes_f32(self._h, _p(raw), n)
        return raw.reshape(n, 16)

    def __del__(self):
        try:
            getattr(lib(), f"oracle_trimesh_free_{self.prec}")(self._h)
        except Exception:
            pass


def _take_pairs(h) -> np.ndarray:
    n = lib().oracle_pairs_count(h)
    out = np.empty((n, 2), dtype=np.uint32)
    if n:
        lib().oracle_pairs_copy(h, _p(out))
    lib().oracle_pairs_free(h)
    return out


class Bvh:
    """Reference Bvh built with BvhBuildStrategy::Binned (f32)."""

    def __init__(self, aabbs: np.ndarray):
        self.a = np.ascontiguousarray(aabbs, dtype=np.float32)
        self._h = lib().oracle_bvh_new_f32(_p(self.a), self.a.shape[0])

    def refit(self, aabbs: np.ndarray) -> None:
        a = np.ascontiguousarray(aabbs, dtype=np.float32)
        lib().oracle_bvh_refit_f32(self._h, _p(a), a.shape[0])

    def nodes(self) -> np.ndarray:
        n = lib().oracle_bvh_nodes_f32(self._h, None, 0)
        raw = np.empty(n * 16, dtype=np.float32)
        lib().oracle_bvh_nodes_f32(self._h, _p(raw), n)
        return raw.reshape(n, 16)

    def traverse_bvtt_single_tree(self) -> np.ndarray:
        """Pairs in the reference's callback order (not canonicalised)."""
        return _take_pairs(lib().oracle_bvh_self_pairs_f32(self._h))

    def leaf_pairs(self, other: "Bvh") -> np.ndarray:
        return _take_pairs(lib().oracle_bvh_leaf_pairs_f32(self._h, other._h))

    def __del__(self):
        try:
            lib().oracle_bvh_free_f32(self._h)
        except Exception:
            pass


def canonical_sorted_pairs(pairs: np.ndarray) -> np.ndarray:
    """(min, max) per row, rows sorted lexicographically."""
    if len(pairs) == 0:
        return pairs.reshape(0, 2)
    a = np.minimum(pairs[:, 0], pairs[:, 1])
    b = np.maximum(pairs[:, 0], pairs[:, 1])
    order = np.lexsort((b, a))
    return np.stack([a[order], b[order]], axis=1)


def sorted_pairs(pairs: np.ndarray) -> np.ndarray:
    if len(pairs) == 0:
        return pairs.reshape(0, 2)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order]


def _shape_arrays(shapes):
    t, prm, pos, pool = shapes.arrays()
    return (np.ascontiguousarray(t, np.uint32), np.ascontiguousarray(prm, np.float32),
            np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(pool, np.float32))


def shape_aabbs(shapes, margin: float = 0.0) -> np.ndarray:
    """Shape::compute_aabb(pos).loosened(margin) for every shape of a parry_gb300.shapes.ShapeSet."""
    t, prm, pos, pool = _shape_arrays(shapes)
    out = np.empty((len(t), 6), np.float32)
    lib().oracle_shape_aabbs_f32(_p(t), _p(prm), _p(pos), _p(pool), len(pool), len(t), float(margin), _p(out))
    return out


def contacts(shapes, pairs: np.ndarray, prediction: float, init_dirs: np.ndarray | None = None, precision: str = "f32",
             threads: int | None = None):
    """query::contact(pos_a, a, pos_b, b, prediction) per (a, b) row of `pairs`.

    Returns (has_contact u8 (k,), out (k, 13) = point1, point2, normal1, normal2, dist, stats dict)."""
    t, prm, pos, pool = _shape_arrays(shapes)
    pairs = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
    k = len(pairs)
    dt = np.float32 if precision == "f32" else np.float64
    out = np.empty((k, 13), dt)
    has = np.empty(k, np.uint8)
    st = np.zeros(7, np.uint64)
    idir = None if init_dirs is None else np.ascontiguousarray(init_dirs, np.float32).reshape(-1, 3)
    getattr(lib(), f"oracle_contacts_{precision}")(_p(t), _p(prm), _p(pos), _p(pool), len(pool), len(t), _p(pairs), k,
                                                   float(prediction), _p(idir), threads if threads is not None else default_threads(),
                                                   _p(out), _p(has), _p(st))
    return has, out, {"gjk_iters": int(st[0]), "epa_iters": int(st[1]), "epa_calls": int(st[2]),
                      "epa_max_faces": int(st[3]), "epa_max_verts": int(st[4]), "epa_max_silhouette": int(st[5]),
                      "support_vertices": int(st[6])}


def cast_shapes(shapes, pairs: np.ndarray, velocities: np.ndarray, max_toi: float = float(np.finfo(np.float32).max),
                target_distance: float = 0.0, stop_at_penetration: bool = True, compute_impact_geometry_on_penetration: bool = True,
                precision: str = "f32", threads: int | None = None):
    """query::cast_shapes(pos_a, vel_a, a, pos_b, vel_b, b, options) per (a, b) row of `pairs`;
    velocities = per-shape linear velocities (n, 3).

    Returns (status u8 (k,) = ShapeCastStatus (0 out of iterations, 1 converged, 2 failed,
    3 penetrating or within target distance) or 255 for None, out (k, 13) = toi, witness1,
    witness2, normal1, normal2, stats dict)."""
    t, prm, pos, pool = _shape_arrays(shapes)
    pairs = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
    vel = np.ascontiguousarray(velocities, np.float32).reshape(-1, 3)
    k = len(pairs)
    dt = np.float32 if precision == "f32" else np.float64
    out = np.empty((k, 13), dt)
    status = np.empty(k, np.uint8)
    st = np.zeros(3, np.uint64)
    opts = np.array([max_toi, target_distance, 1.0 if stop_at_penetration else 0.0,
                     1.0 if compute_impact_geometry_on_penetration else 0.0], np.float32)
    getattr(lib(), f"oracle_cast_shapes_{precision}")(_p(t), _p(prm), _p(pos), _p(pool), len(pool), len(t), _p(pairs), k, _p(vel),
                                                      _p(opts), threads if threads is not None else default_threads(), _p(out),
                                                      _p(status), _p(st))
    return status, out, {"gjk_iters": int(st[0]), "epa_iters": int(st[1]), "epa_calls": int(st[2])}


class _PolyIn(C.Structure):
    """Field layout of the library's parrygpu_polyhedra (ConvexPolyhedron topology)."""
    _fields_ = [("n_hulls", U64), ("hulls", P), ("n_faces", U64), ("face_normals", P), ("face_ranges", P),
                ("n_face_entries", U64), ("face_vertices", P), ("face_edges", P), ("vertex_ranges", P),
                ("n_vertex_entries", U64), ("vertex_faces", P), ("vertex_edges", P), ("n_edges", U64), ("edge_dirs", P)]


def _poly_struct(shapes):
    """(pointer to a _PolyIn or None, keep-alive) for a ShapeSet's hull topology."""
    poly = shapes.polyhedra() if hasattr(shapes, "polyhedra") else None
    if poly is None:
        return None, None
    hulls, topo = poly
    arrs = {"hulls": np.ascontiguousarray(hulls, np.uint32)}
    for key, val in topo.items():
        arrs[key] = np.ascontiguousarray(val, np.float32 if key in ("face_normals", "edge_dirs") else np.uint32)
    ptr = {key: (a.ctypes.data if a.size else None) for key, a in arrs.items()}
    st = _PolyIn(len(arrs["hulls"]), ptr["hulls"], len(arrs["face_normals"]), ptr["face_normals"], ptr["face_ranges"],
                 len(arrs["face_vertices"]), ptr["face_vertices"], ptr["face_edges"], ptr["vertex_ranges"],
                 len(arrs["vertex_faces"]), ptr["vertex_faces"], ptr["vertex_edges"], len(arrs["edge_dirs"]), ptr["edge_dirs"])
    return C.cast(C.pointer(st), C.c_void_p), (st, arrs)


MANIFOLD_MAX_POINTS = 24
MANIFOLD_WORDS = 8 + 10 * MANIFOLD_MAX_POINTS


def empty_manifolds(k: int) -> np.ndarray:
    """k zeroed manifold records (uint32 words, the parrygpu_manifold layout): ContactManifold::new()."""
    return np.zeros((k, MANIFOLD_WORDS), np.uint32)


def contact_manifolds(shapes, pairs: np.ndarray, prediction: float, records: np.ndarray, threads: int | None = None,
                      pseudo: np.ndarray | None = None, pseudo_first: int = 0, init_dirs: np.ndarray | None = None) -> dict:
    """DefaultQueryDispatcher::contact_manifold_convex_convex(pos_a^-1 pos_b, a, b, c_a, c_b, prediction,
    manifold) for every (a, b) row of `pairs`, updating `records` (k x MANIFOLD_WORDS uint32) in
    place. Normal constraints c: a triangle shape of index >= pseudo_first whose params word 2 holds
    j > 0 uses row j - 1 of `pseudo` (rows of 12 floats: face, e01, e12, e20); else None.
    init_dirs (k x 3 float32, optional): the polyhedral generator's GJK start direction for a pair
    whose record holds no cached normal (contact_manifolds_pfm_pfm.rs:67-76 otherwise starts from the
    relative translation); a row that does not normalise keeps that default."""
    if init_dirs is not None:
        init_dirs = np.ascontiguousarray(init_dirs, np.float32).reshape(-1, 3)
        assert len(init_dirs) == len(pairs)
    if pseudo is not None:
        pseudo = np.ascontiguousarray(pseudo, np.float32).reshape(-1, 12)
    t, prm, pos, pool = _shape_arrays(shapes)
    pairs = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
    k = len(pairs)
    assert records.dtype == np.uint32 and records.shape == (k, MANIFOLD_WORDS) and records.flags.c_contiguous
    st = np.zeros(5, np.uint64)
    poly, keep = _poly_struct(shapes)
    lib().oracle_manifolds_f32(_p(t), _p(prm), _p(pos), _p(pool), len(pool), len(t), poly, _p(pairs), k, float(prediction),
                               threads if threads is not None else default_threads(), _p(records), _p(st),
                               _p(pseudo) if pseudo is not None and len(pseudo) else None, int(pseudo_first),
                               _p(init_dirs) if init_dirs is not None else None)
    del keep
    return {"gjk_iters": int(st[0]), "epa_iters": int(st[1]), "epa_calls": int(st[2]), "unsupported": int(st[3]),
            "max_points": int(st[4])}


def trimesh_pseudo_normals(vertices: np.ndarray, indices: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """TriMesh::triangle_normal_constraints of every triangle of a mesh built with
    TriMeshFlags::FIX_INTERNAL_EDGES (trimesh.rs:1251-1320, 1348-1407, 1911-1931): (nt, 12) f32 rows
    (face, e01, e12, e20) and a (nt,) bool mask of the triangles that have constraints."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    i = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
    out = np.zeros((len(i), 12), np.float32)
    ok = np.zeros(len(i), np.uint8)
    lib().oracle_trimesh_pseudo_normals_f32(_p(v), len(v), _p(i), len(i), _p(out), _p(ok))
    return out, ok.astype(bool)


def project_local_normals(pseudo: np.ndarray, dirs: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """TrianglePseudoNormals::project_local_normal (triangle_pseudo_normals.rs:35-99) per row:
    (projected directions (n, 3), ok mask) - ok False is the reference's None."""
    pn = np.ascontiguousarray(pseudo, np.float32).reshape(-1, 12)
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    assert len(pn) == len(d)
    out = np.zeros_like(d)
    ok = np.zeros(len(d), np.uint8)
    lib().oracle_project_local_normals_f32(_p(pn), _p(d), len(d), _p(out), _p(ok))
    return out, ok.astype(bool)


def inv_mul(pose1: np.ndarray, poses2: np.ndarray) -> np.ndarray:
    """Isometry::inv_mul: pose1^-1 * pose2 for each row of poses2 (pose7, f32)."""
    p1 = np.ascontiguousarray(pose1, np.float32).reshape(7)
    p2 = np.ascontiguousarray(poses2, np.float32).reshape(-1, 7)
    out = np.empty_like(p2)
    lib().oracle_inv_mul_f32(_p(p1), _p(p2), len(p2), _p(out))
    return out


def _with_triangles(shapes, tri_vertices: np.ndarray, mesh_pose: np.ndarray, constrained: np.ndarray | None = None):
    """The shapes followed by one Triangle shape per mesh triangle (vertices appended to the pool,
    posed at the mesh pose): triangle t has shape index n + t; with `constrained` (mask), params
    word 2 of triangle t is t + 1 where it has normal constraints (row t of the table)."""
    from parry_gb300.shapes import ShapeSet, TRIANGLE
    t, prm, pos, pool = shapes.arrays()
    n, nt = len(t), len(tri_vertices)
    first = np.arange(nt, dtype=np.uint32) * 3 + np.uint32(len(pool))
    tp = np.zeros((nt, 4), np.float32)
    tp.view(np.uint32)[:, 0] = first
    tp.view(np.uint32)[:, 1] = 3
    if constrained is not None:
        tp.view(np.uint32)[:, 2] = np.where(constrained, np.arange(1, nt + 1, dtype=np.uint32), 0)
    poly = shapes.polyhedra()
    if poly is not None:
        hulls, topo = poly
        topo = dict(topo)
        topo["vertex_ranges"] = np.concatenate([topo["vertex_ranges"], np.zeros((3 * nt, 2), np.uint32)])
        poly = (hulls, topo)
    return ShapeSet.from_arrays(np.concatenate([t, np.full(nt, TRIANGLE, np.uint32)]), np.concatenate([prm, tp]),
                                np.concatenate([pos, np.repeat(np.asarray(mesh_pose, np.float32).reshape(1, 7), nt, 0)]),
                                np.concatenate([pool, tri_vertices.reshape(-1, 3)]), poly)


class TriMeshContacts:
    """contact_manifolds_trimesh_shape (contact_manifolds_trimesh_shape.rs:82-228) for each shape of a
    set against one TriMesh (the mesh is shape 1), frame after frame; with fix_internal_edges
    (TriMeshFlags::FIX_INTERNAL_EDGES) each triangle's TrianglePseudoNormals constrain the normals, with the reference's workspace: the shape's AABB in the mesh frame loosened by
    the prediction, kept while it still contains the new one (else enlarged by min(extent / 10, 0.1)
    per axis and the triangles whose AABBs intersect it queried again), and one ContactManifold per
    interfering triangle carried over by triangle id. Interferences are kept in ascending triangle
    order: the reference's carry-over loop walks old and new lists as sorted lists, and its BVH
    returns them in tree order, which depends on the tree (a deviation recorded as D-8)."""

    def __init__(self, vertices: np.ndarray, indices: np.ndarray, n_shapes: int, fix_internal_edges: bool = False):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        self.pseudo, self.constrained = trimesh_pseudo_normals(v, i) if fix_internal_edges else (None, None)
        self.tri = np.ascontiguousarray(v[i], np.float32)  # (nt, 3, 3)
        # aabb_triangle.rs: a.min(b).min(c), a.max(b).max(c)
        self.tri_min = np.minimum(np.minimum(self.tri[:, 0], self.tri[:, 1]), self.tri[:, 2])
        self.tri_max = np.maximum(np.maximum(self.tri[:, 0], self.tri[:, 1]), self.tri[:, 2])
        # Sweep index on x: triangles sorted by their AABB's min x; a query [lo, hi] on x can only
        # meet triangles whose min x lies in [lo - widest x extent, hi]. The answer is the same set
        # of triangles as the reference's BVH query (AABB intersection), found faster.
        self.sweep = np.argsort(self.tri_min[:, 0], kind="stable")
        self.sweep_x = self.tri_min[self.sweep, 0]
        self.widest_x = float((self.tri_max[:, 0] - self.tri_min[:, 0]).max()) if len(self.tri) else 0.0
        big = np.float32(np.finfo(np.float32).max)
        self.aabb = np.concatenate([np.full((n_shapes, 3), big, np.float32), np.full((n_shapes, 3), -big, np.float32)], 1)
        self.inter = [np.zeros(0, np.uint32) for _ in range(n_shapes)]
        self.records = [empty_manifolds(0) for _ in range(n_shapes)]

    def update(self, mesh_pose: np.ndarray, shapes, prediction: float, threads: int | None = None) -> dict:
        t, prm, pos, pool = shapes.arrays()
        n = len(t)
        rel = inv_mul(mesh_pose, pos)
        nb = shape_aabbs(shapes.with_poses(rel), prediction)  # compute_aabb(pos12).loosened(prediction)
        f0, f1 = np.float32(0.1), np.float32(10.0)
        for s in range(n):
            mins, maxs = nb[s, :3].copy(), nb[s, 3:].copy()
            same = bool(np.all(self.aabb[s, :3] <= mins) and np.all(self.aabb[s, 3:] >= maxs))
            if same:
                continue
            extra = np.minimum((maxs - mins) / f1, f0)
            mins, maxs = mins - extra, maxs + extra
            a = np.searchsorted(self.sweep_x, np.float64(mins[0]) - self.widest_x, "left")
            b = np.searchsorted(self.sweep_x, maxs[0], "right")
            cand = self.sweep[a:b]
            hit = np.all(self.tri_min[cand] <= maxs, 1) & np.all(self.tri_max[cand] >= mins, 1)
            new = np.sort(cand[hit]).astype(np.uint32)
            old, old_rec = self.inter[s], self.records[s]
            rec = empty_manifolds(len(new))
            j = np.searchsorted(old, new)
            found = (j < len(old)) & (old[np.minimum(j, max(len(old) - 1, 0))] == new) if len(old) else np.zeros(len(new), bool)
            rec[found] = old_rec[j[found]]
            self.inter[s], self.records[s] = new, rec
            self.aabb[s, :3], self.aabb[s, 3:] = mins, maxs
        combined = _with_triangles(shapes, self.tri, mesh_pose, self.constrained)
        counts = [len(x) for x in self.inter]
        if sum(counts) == 0:
            return {"pairs": 0}
        pairs = np.concatenate([np.stack([self.inter[s] + np.uint32(n), np.full(counts[s], s, np.uint32)], 1)
                                for s in range(n) if counts[s]]).astype(np.uint32)
        recs = np.ascontiguousarray(np.concatenate([self.records[s] for s in range(n) if counts[s]]))
        st = contact_manifolds(combined, pairs, prediction, recs, threads, self.pseudo, n)
        k = 0
        for s in range(n):
            self.records[s] = recs[k:k + counts[s]].copy()
            k += counts[s]
        st["pairs"] = int(len(pairs))
        return st


class Compound:
    """Reference Compound (shape set): binned BVH over part AABBs, RayCast with part poses."""

    def __init__(self, shapes, precision: str = "f32"):
        self.arr = _shape_arrays(shapes)
        t, prm, pos, pool = self.arr
        self.prec = precision
        self._h = getattr(lib(), f"oracle_compound_new_{precision}")(_p(t), _p(prm), _p(pos), _p(pool), len(pool), len(t))

    def cast_rays_and_get_normal(self, rays: np.ndarray, max_toi: float, solid: bool = True, pose=None, lowest_index: bool = True,
                                 threads: int | None = None, want_stats: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        dt = np.float32 if self.prec == "f32" else np.float64
        part = np.empty(n, np.uint32)
        toi = np.empty(n, dt)
        nrm = np.empty((n, 3), dt)
        st = np.zeros(2, np.uint64)
        pz = None if pose is None else np.ascontiguousarray(pose, np.float32)
        getattr(lib(), f"oracle_compound_cast_rays_{self.prec}")(self._h, _p(pz), _p(rays), n, float(max_toi), 1 if solid else 0,
                                                                 1 if lowest_index else 0,
                                                                 threads if threads is not None else default_threads(),
                                                                 _p(part), _p(toi), _p(nrm), _p(st) if want_stats else None)
        if want_stats:
            return part, toi, nrm, {"wide_visits": int(st[0]), "leaf_tests": int(st[1])}
        return part, toi, nrm

    def __del__(self):
        try:
            getattr(lib(), f"oracle_compound_free_{self.prec}")(self._h)
        except Exception:
            pass


def integrate(poses: np.ndarray, velocities: np.ndarray, dt: float) -> np.ndarray:
    """One pose-integration step of the frame pipeline (decision D-5), f32; returns new poses."""
    out = np.ascontiguousarray(poses, np.float32).copy()
    vel = np.ascontiguousarray(velocities, np.float32)
    lib().oracle_integrate_f32(_p(out), _p(vel), len(out), float(dt))
    return out


def scene_frames(shapes, velocities: np.ndarray, prediction: float, dt: float, frames: int, rays: np.ndarray | None = None,
                 max_toi: float = 100.0, threads: int | None = None, dirs_fn=None) -> dict:
    """The frame pipeline restated with the oracle pieces: integrate, AABBs loosened by prediction / 2,
    binned-BVH self pairs, contact manifolds kept per pair across frames (new pairs start empty), and
    the rays cast against the final frame's shapes (Compound semantics, lowest index on ties).
    dirs_fn(shapes, pairs) -> (k x 3) (optional) gives each frame's GJK start directions for the
    pairs without a cached normal (the learned seeding; contact_manifolds' init_dirs).
    Returns poses, sorted pairs, their manifold words, and the ray results."""
    poses = np.ascontiguousarray(shapes.arrays()[2], np.float32).copy()
    records: dict = {}
    pairs = np.zeros((0, 2), np.uint32)
    recs = np.zeros((0, MANIFOLD_WORDS), np.uint32)
    s = shapes
    for _ in range(frames):
        poses = integrate(poses, velocities, dt)
        s = shapes.with_poses(poses)
        aabbs = shape_aabbs(s, 0.5 * prediction)
        pairs = canonical_sorted_pairs(Bvh(aabbs).traverse_bvtt_single_tree()) if len(aabbs) > 1 else np.zeros((0, 2), np.uint32)
        recs = np.zeros((len(pairs), MANIFOLD_WORDS), np.uint32)
        for i, (a, b) in enumerate(pairs):
            old = records.get((int(a), int(b)))
            if old is not None:
                recs[i] = old
        dirs = dirs_fn(s, pairs) if dirs_fn is not None and len(pairs) else None
        contact_manifolds(s, pairs, prediction, recs, threads=threads, init_dirs=dirs)
        records = {(int(a), int(b)): recs[i].copy() for i, (a, b) in enumerate(pairs)}
    out = {"poses": poses, "pairs": pairs, "manifolds": recs}
    if rays is not None:
        c = Compound(s)
        part, toi, nrm = c.cast_rays_and_get_normal(rays, max_toi, solid=True, threads=threads)
        out.update(ray_part=part, ray_toi=toi, ray_normal=nrm)
    return out
