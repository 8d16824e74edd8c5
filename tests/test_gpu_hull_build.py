"""ConvexPolyhedron::from_convex_hull on the GPU (parrygpu_polyhedra_build_gpu).

Pinned on the reference: the two clouds of parry's own convex-hull tests
(crates/parry3d/tests/geometry/convex_hull.rs, fixtures in tests/golden/convex_hull_fixtures.npz)
and a sample of the measured workload's clouds must give triangulations that the oracle's
restatement of transformation::check_convex_hull accepts, with every hull vertex a cloud point and
no cloud point above a hull triangle; the ConvexPolyhedron of clouds in general position passes the
face checks (points below every face plane, convex counter-clockwise faces, V - E + F = 2). Against
the host builder: the same bytes for every output array, on ellipsoid clouds of 16-64 and 8-256
points and on degenerate clouds (coplanar, collinear, repeated points, cube corners with coplanar
faces)."""
from pathlib import Path

import numpy as np
import pytest

from oracle.hull_check import check_convex_hull, check_convex_hulls, polyhedron_properties, triangulation_properties
from parry_gb300 import workloads as W
from parry_gb300.polyhedra import build_polyhedra

pytestmark = pytest.mark.gpu
FIXTURES = Path(__file__).resolve().parent / "golden" / "convex_hull_fixtures.npz"


def _special_clouds():
    rng = np.random.default_rng(0)
    clouds = [np.zeros((4, 3)), np.c_[rng.uniform(size=(10, 2)), np.zeros(10)], np.outer(np.arange(6), [1, 2, 3]),
              np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], float),
              np.repeat(rng.uniform(size=(5, 3)), 3, axis=0), rng.uniform(size=(40, 3)), rng.normal(size=(300, 3)),
              np.array([[x, y, z] for x in (0, 1, 2) for y in (0, 1, 2) for z in (0, 1, 2)], float), rng.uniform(size=(3, 3))]
    cloud = np.concatenate(clouds).astype(np.float32)
    count = np.array([len(c) for c in clouds], np.uint32)
    first = np.concatenate([[0], np.cumsum(count)[:-1]]).astype(np.uint32)
    return cloud, first, count


@pytest.mark.parametrize("case", ["16-64", "8-256", "special"])
def test_gpu_build_equals_host_build(gpu_ctx, case):
    if case == "special":
        cloud, first, count = _special_clouds()
    else:
        lo, hi = (16, 64) if case == "16-64" else (8, 256)
        cloud, first, count = W.ellipsoid_hulls(20000 if lo == 16 else 3000, 50 + lo, 7, lo, hi)
    host = build_polyhedra(cloud, first, count, with_triangles=True)
    dev = build_polyhedra(cloud, first, count, ctx=gpu_ctx, with_triangles=True)
    np.testing.assert_array_equal(dev[0].view(np.uint32), host[0].view(np.uint32))
    np.testing.assert_array_equal(dev[1], host[1])
    for k in host[2]:
        np.testing.assert_array_equal(dev[2][k].view(np.uint32), host[2][k].view(np.uint32), err_msg=k)
    if case != "special":
        assert host[1][:, 6].all()
    else:
        assert host[1][:, 6].sum() >= 4 and not host[1][:, 6].all()


def test_gpu_build_rejects_out_of_range(gpu_ctx):
    import parry_gb300 as pg
    cloud = np.zeros((10, 3), np.float32)
    with pytest.raises(pg.ParryGpuError):
        build_polyhedra(cloud, np.array([5], np.uint32), np.array([8], np.uint32), ctx=gpu_ctx)


@pytest.mark.parametrize("name", ["complex", "planar"])
def test_reference_fixtures_pass_check_convex_hull(gpu_ctx, name):
    cloud = np.load(FIXTURES)[name]
    one = np.array([0], np.uint32)
    points, hulls, topo = build_polyhedra(cloud, one, np.array([len(cloud)], np.uint32), ctx=gpu_ctx, with_triangles=True)
    assert hulls[0, 6] == 1
    t0, nt = topo["tri_ranges"][0]
    tris = topo["triangles"][t0:t0 + nt]
    check_convex_hull(points[:hulls[0, 1]], tris)
    assert triangulation_properties(cloud, points[:hulls[0, 1]], tris) == []
    if name == "planar":
        assert hulls[0, 3] == 2
        assert polyhedron_properties(cloud, one, [len(cloud)], points, hulls, topo, [0]) == []


def test_workload_sample_passes_check_convex_hull(gpu_ctx):
    """65,536 clouds of the hull-construction workload (16-64 points on ellipsoids, the bench's
    generator) and 4,096 of 8-256 points: every triangulation passes check_convex_hull; a subsample
    also passes the triangulation and ConvexPolyhedron checks."""
    for n, lo, hi in ((65536, 16, 64), (4096, 8, 256)):
        cloud, first, count = W.ellipsoid_hulls(n, 66, 7, lo, hi)
        points, hulls, topo = build_polyhedra(cloud, first, count, ctx=gpu_ctx, with_triangles=True)
        assert hulls[:, 6].all()
        ok = check_convex_hulls(points, hulls, topo["tri_ranges"], topo["triangles"])
        assert ok.all(), f"{int((~ok).sum())} hulls fail check_convex_hull"
        sub = range(0, n, 257)
        assert polyhedron_properties(cloud, first, count, points, hulls, topo, sub) == []
        for h in sub:
            t0, nt = topo["tri_ranges"][h]
            p = points[hulls[h, 0]:hulls[h, 0] + hulls[h, 1]]
            assert triangulation_properties(cloud[first[h]:first[h] + count[h]], p, topo["triangles"][t0:t0 + nt]) == []


def test_gpu_build_into_caller_buffers(gpu_ctx):
    """build_polyhedra(out=...) into larger pinned buffers returns views of their leading rows that
    equal the arrays of a plain build, byte for byte; a buffer too short is refused."""
    import torch
    cloud, first, count = W.ellipsoid_hulls(3000, 66, 7, 16, 64)
    pts, hulls, topo = build_polyhedra(cloud, first, count, ctx=gpu_ctx)

    def pinned(rows, cols, dt):
        shape = (rows + 17, cols) if cols else (rows + 17,)
        return torch.zeros(shape, dtype=dt, pin_memory=True).numpy()
    out = {"points": pinned(len(pts), 3, torch.float32), "hulls": pinned(len(hulls), 8, torch.int32).view(np.uint32)}
    for k, a in topo.items():
        out[k] = pinned(len(a), a.shape[1] if a.ndim == 2 else 0, torch.float32 if a.dtype == np.float32 else torch.int32)
        if a.dtype == np.uint32:
            out[k] = out[k].view(np.uint32)
    p2, h2, t2 = build_polyhedra(cloud, first, count, ctx=gpu_ctx, out=out)
    np.testing.assert_array_equal(p2.view(np.uint32), pts.view(np.uint32))
    np.testing.assert_array_equal(h2, hulls)
    for k in topo:
        np.testing.assert_array_equal(t2[k].view(np.uint32), topo[k].view(np.uint32))
        assert np.shares_memory(t2[k], out[k])
    short = dict(out)
    short["face_vertices"] = out["face_vertices"][: len(topo["face_vertices"]) - 1]
    with pytest.raises(ValueError):
        build_polyhedra(cloud, first, count, ctx=gpu_ctx, out=short)
