"""transformation::check_convex_hull restated in the oracle, pinned on hand-made meshes, and the
reference's own convex-hull fixtures (crates/parry3d/tests/geometry/convex_hull.rs: a 4,054-point
cloud with repeated points, and 8 coplanar points) through the library's host hull builder: the
triangulation passes check_convex_hull and the ConvexPolyhedron passes the build-independent
checks (triangulation: hull vertices are cloud points, no cloud point above a hull triangle; the
ConvexPolyhedron's own checks on the planar cloud, whose facets are exactly coplanar). The GPU
builder runs the same fixtures in tests/test_gpu_hull_build.py."""
from pathlib import Path

import numpy as np
import pytest

from oracle.hull_check import (ConvexHullError, check_convex_hull, check_convex_hulls, polyhedron_properties,
                               triangulation_properties)

FIXTURES = Path(__file__).resolve().parent / "golden" / "convex_hull_fixtures.npz"
TET = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
TET_TRIS = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [2, 0, 3]], np.uint32)


def test_check_convex_hull_rules():
    check_convex_hull(TET, TET_TRIS)
    with pytest.raises(ConvexHullError, match="DuplicatePoints"):
        check_convex_hull(np.concatenate([TET, TET[1:2]]), TET_TRIS)
    with pytest.raises(ConvexHullError, match="UnfinishedTriangle"):
        check_convex_hull(TET, TET_TRIS[:3])
    with pytest.raises(ConvexHullError, match="TJunction"):
        check_convex_hull(np.concatenate([TET, [[1, 1, 1]]]), np.concatenate([TET_TRIS, [[0, 1, 4]]]))
    with pytest.raises(ConvexHullError, match="repeats a vertex"):
        check_convex_hull(TET, np.concatenate([TET_TRIS, [[0, 0, 1]]]))
    # a closed surface of the wrong genus: two tetrahedra sharing only a vertex
    two = np.concatenate([TET, TET[1:] + 2.0])
    tris = np.concatenate([TET_TRIS, np.where(TET_TRIS == 0, 0, TET_TRIS + 3)])
    with pytest.raises(ConvexHullError, match="Euler"):
        check_convex_hull(two, tris)


def _host_build(cloud):
    from parry_gb300.polyhedra import build_polyhedra
    return build_polyhedra(cloud, np.array([0], np.uint32), np.array([len(cloud)], np.uint32), threads=1, with_triangles=True)


@pytest.mark.parametrize("name", ["complex", "planar"])
def test_reference_fixtures_host_builder(name):
    cloud = np.load(FIXTURES)[name]
    points, hulls, topo = _host_build(cloud)
    assert hulls[0, 6] == 1, "ConvexPolyhedron::from_convex_hull gave no topology"
    t0, nt = topo["tri_ranges"][0]
    tris = topo["triangles"][t0:t0 + nt]
    check_convex_hull(points[:hulls[0, 1]], tris)
    assert triangulation_properties(cloud, points[:hulls[0, 1]], tris) == []
    if name == "planar":
        assert hulls[0, 3] == 2  # the two sides of the polygon
        assert polyhedron_properties(cloud, [0], [len(cloud)], points, hulls, topo, [0]) == []


def test_batch_check_agrees_with_scalar_check():
    from parry_gb300 import workloads as W
    from parry_gb300.polyhedra import build_polyhedra
    cloud, first, count = W.ellipsoid_hulls(300, 77, 7, 4, 64)
    points, hulls, topo = build_polyhedra(cloud, first, count, threads=2, with_triangles=True)
    ok = check_convex_hulls(points, hulls, topo["tri_ranges"], topo["triangles"])
    assert ok.all()
    for h in range(0, 300, 37):
        t0, nt = topo["tri_ranges"][h]
        check_convex_hull(points[hulls[h, 0]:hulls[h, 0] + hulls[h, 1]], topo["triangles"][t0:t0 + nt])
    # a broken triangulation is caught by both
    bad = topo["triangles"].copy()
    t0 = topo["tri_ranges"][5, 0]
    bad[t0, 1] = bad[t0, 2]
    assert not check_convex_hulls(points, hulls, topo["tri_ranges"], bad)[5]
    assert polyhedron_properties(cloud, first, count, points, hulls, topo, range(0, 300, 7)) == []
