"""ConvexPolyhedron::from_convex_hull on the GPU (parrygpu_polyhedra_build_gpu) against the host
builder: the same bytes for every output array, on ellipsoid clouds of 16-64 and 8-256 points and
on degenerate clouds (coplanar, collinear, repeated points, cube corners with coplanar faces)."""
import numpy as np
import pytest

from parry_gb300 import workloads as W
from parry_gb300.polyhedra import build_polyhedra

pytestmark = pytest.mark.gpu


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
    host = build_polyhedra(cloud, first, count)
    dev = build_polyhedra(cloud, first, count, ctx=gpu_ctx)
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
