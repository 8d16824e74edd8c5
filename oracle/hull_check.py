"""Oracle (test infrastructure only): parry's validation of a convex hull, restated.

check_convex_hull follows transformation::check_convex_hull
(src/transformation/convex_hull3/validation.rs:33-108, paths relative to the parry repository):
no two points equal; no triangle repeats a vertex (an assert there); every edge, as an unordered
pair, borders exactly two triangles (a third one is a `TJunction`, a single one an
`UnfinishedTriangle`); and the Euler characteristic V + F - E = 2 (an assert there). It is the check
the reference's own tests apply to `transformation::convex_hull` (crates/parry3d/tests/geometry/
convex_hull.rs).

check_convex_hulls applies the same rules to many hulls at once (numpy over all triangles).
triangulation_properties adds checks that do not depend on how a hull was built: every hull vertex
is one of its cloud's points and every cloud point lies on or below the plane of every hull
triangle. polyhedron_properties checks the ConvexPolyhedron that from_convex_mesh makes of a hull
(src/shape/convex_polyhedron.rs:390-639): every cloud point on or below every face plane, every face
convex and counter-clockwise about its normal, V - E + F = 2 over its faces and their edges. That
holds when no two adjacent hull triangles are within from_convex_mesh's merge angle of coplanar
without being coplanar (points in general position, or exactly coplanar facets); on clouds with
many nearly coplanar triangles the reference's merge can join triangles into faces that are not
planar or not simply connected, so only the triangulation checks apply there.
"""
from __future__ import annotations

import numpy as np


class ConvexHullError(AssertionError):
    pass


def check_convex_hull(points: np.ndarray, triangles: np.ndarray) -> None:
    """Raises ConvexHullError naming the first rule the (points, triangles) mesh breaks."""
    points = np.asarray(points)
    triangles = np.asarray(triangles, np.int64).reshape(-1, 3)
    n = len(points)
    for i in range(n):  # DuplicatePoints(i, j): the first pair in (i, j) order
        same = np.nonzero(np.all(points[i + 1:] == points[i], axis=1))[0]
        if len(same):
            raise ConvexHullError(f"DuplicatePoints({i}, {i + 1 + int(same[0])})")
    edges: dict = {}
    for itri, tri in enumerate(triangles):
        if tri[0] == tri[1] or tri[0] == tri[2] or tri[2] == tri[1]:
            raise ConvexHullError(f"triangle {itri} repeats a vertex")
        for i in range(3):
            a, b = int(tri[i]), int(tri[(i + 1) % 3])
            key = (min(a, b), max(a, b))
            adj = edges.get(key)
            if adj is None:
                edges[key] = [itri, None]
            elif adj[1] is not None:
                raise ConvexHullError(f"TJunction({itri}, {a}, {b})")
            else:
                adj[1] = itri
    if any(adj[1] is None for adj in edges.values()):
        raise ConvexHullError("UnfinishedTriangle")
    if n + len(triangles) - len(edges) != 2:
        raise ConvexHullError(f"Euler characteristic {n + len(triangles) - len(edges)} != 2")


def check_convex_hulls(points: np.ndarray, hulls: np.ndarray, tri_ranges: np.ndarray, triangles: np.ndarray,
                       which: np.ndarray | None = None) -> np.ndarray:
    """check_convex_hull's rules for every hull h in `which` (default: all) of a batch: hull h's points
    are points[hulls[h, 0] : + hulls[h, 1]], its triangles triangles[tri_ranges[h, 0] : + tri_ranges[h, 1]]
    with hull-local ids. Returns a bool array (True = the hull passes)."""
    hulls = np.asarray(hulls, np.int64)
    tri_ranges = np.asarray(tri_ranges, np.int64)
    if which is None:
        which = np.arange(len(hulls))
    ok = np.ones(len(which), bool)
    # triangles of the selected hulls, with the hull's slot in `which`
    counts = tri_ranges[which, 1]
    slot = np.repeat(np.arange(len(which)), counts)
    starts = np.repeat(tri_ranges[which, 0] - np.concatenate([[0], np.cumsum(counts)[:-1]]), counts)
    tri = np.asarray(triangles, np.int64)[np.arange(counts.sum()) + starts]
    nv = hulls[which, 1]
    ok &= counts > 0
    bad = (tri[:, 0] == tri[:, 1]) | (tri[:, 0] == tri[:, 2]) | (tri[:, 1] == tri[:, 2]) | (tri >= nv[slot][:, None]).any(1)
    ok[np.unique(slot[bad])] = False
    # every undirected edge exactly twice
    a = tri[:, [0, 1, 2]].reshape(-1)
    b = tri[:, [1, 2, 0]].reshape(-1)
    es = np.repeat(slot, 3)
    key = (es << 40) | (np.minimum(a, b) << 20) | np.maximum(a, b)
    uk, cnt = np.unique(key, return_counts=True)
    ok[np.unique(uk[cnt != 2] >> 40)] = False
    n_edges = np.bincount(uk >> 40, minlength=len(which))
    ok &= nv + counts - n_edges == 2
    # no two equal points within a hull
    pts = np.asarray(points)
    for s, h in enumerate(which):
        if ok[s]:
            p = pts[hulls[h, 0]:hulls[h, 0] + hulls[h, 1]]
            ok[s] = len(np.unique(p.view(np.uint32).reshape(-1, 3), axis=0)) == len(p)
    return ok


def triangulation_properties(cloud: np.ndarray, points: np.ndarray, triangles: np.ndarray, rel_tol: float = 1e-6) -> list[str]:
    """Build-independent checks of one hull triangulation (hull-local `triangles` into `points`)."""
    fails = []
    c32 = np.asarray(cloud, np.float32)
    cset = {tuple(r) for r in c32.view(np.uint32).reshape(-1, 3)}
    if not all(tuple(r) in cset for r in np.asarray(points, np.float32).view(np.uint32).reshape(-1, 3)):
        fails.append("a hull vertex is not a cloud point")
    c = c32.astype(np.float64)
    p = np.asarray(points, np.float64)
    t = np.asarray(triangles, np.int64).reshape(-1, 3)
    a, b, d = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    n = np.cross(b - a, d - a)
    ln = np.linalg.norm(n, axis=1)
    if (ln == 0).any():
        fails.append(f"{int((ln == 0).sum())} degenerate triangles")
        return fails
    n /= ln[:, None]
    scale = float(np.ptp(c, axis=0).max()) or 1.0
    for k in range(0, len(t), 4096):
        above = (c @ n[k:k + 4096].T) - np.sum(n[k:k + 4096] * a[k:k + 4096], axis=1)[None, :]
        if above.max() > rel_tol * scale:
            fails.append(f"a cloud point lies {above.max():.3g} above a hull triangle")
            break
    return fails


def polyhedron_properties(cloud: np.ndarray, first: np.ndarray, count: np.ndarray, points: np.ndarray, hulls: np.ndarray,
                          topo: dict, which, rel_tol: float = 1e-5) -> list[str]:
    """Build-independent checks of ConvexPolyhedron h for h in `which`; returns failure messages."""
    fails = []
    fn, fr, fv, fe = topo["face_normals"], topo["face_ranges"], topo["face_vertices"], topo["face_edges"]
    for h in which:
        c = np.asarray(cloud[first[h]:first[h] + count[h]], np.float64)
        p0, nv, f0, nf, e0, ne, ok = (int(x) for x in hulls[h, :7])
        if not ok:
            fails.append(f"hull {h}: no topology")
            continue
        p = np.asarray(points[p0:p0 + nv], np.float64)
        scale = float(np.abs(c).max()) or 1.0
        cset = {tuple(r) for r in np.asarray(cloud[first[h]:first[h] + count[h]], np.float32).view(np.uint32)}
        if not all(tuple(r) in cset for r in np.asarray(points[p0:p0 + nv], np.float32).view(np.uint32)):
            fails.append(f"hull {h}: a hull vertex is not a cloud point")
        used_edges = set()
        for f in range(f0, f0 + nf):
            start, num = int(fr[f, 0]), int(fr[f, 1])
            ids = fv[start:start + num].astype(np.int64)
            used_edges.update(int(e) for e in fe[start:start + num])
            n = np.asarray(fn[f], np.float64)
            q = p[ids]
            dist = (c - q[0]) @ n
            if dist.max() > rel_tol * scale:
                fails.append(f"hull {h} face {f - f0}: a cloud point lies {dist.max():.3g} above the face plane")
            # convex, counter-clockwise about the normal
            for k in range(num):
                e1, e2 = q[(k + 1) % num] - q[k], q[(k + 2) % num] - q[(k + 1) % num]
                if np.cross(e1, e2) @ n < -rel_tol * scale * scale:
                    fails.append(f"hull {h} face {f - f0}: not convex counter-clockwise at corner {k}")
                    break
        if nv - len(used_edges) + nf != 2:
            fails.append(f"hull {h}: V - E + F = {nv - len(used_edges) + nf}")
    return fails
