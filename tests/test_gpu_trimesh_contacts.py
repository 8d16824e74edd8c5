"""Contact manifolds of shapes against a TriMesh (contact_manifolds_trimesh_shape) on the GPU against
the oracle, over frames: the interfering triangles of every shape and the record of each
(triangle, shape) manifold bit-exact, with the workspace's AABB kept, enlarged and re-queried as the
shapes move."""
import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import manifold as M
from parry_gb300 import workloads as W
from parry_gb300.shapes import ShapeSet
from tests.test_gpu_manifolds import assert_records_equal

pytestmark = pytest.mark.gpu


def _scene(n_pairs, seed, nx=48, nz=24):
    v, i = W.terrain_mesh(nx, nz, seed=seed)
    t, prm, pos, pool, poly, _ = W.primitive_pairs(n_pairs, seed=seed + 1)
    n = len(t)
    rng = np.random.default_rng(seed)
    pos = pos.copy()
    pos[:, 4] = rng.uniform(1, nx - 1, n)
    pos[:, 6] = rng.uniform(1, nz - 1, n)
    pos[:, 5] = rng.uniform(0.5, 5.0, n)
    vel = rng.normal(size=(n, 3)).astype(np.float32) * np.float32(0.05)
    vel[:, 1] -= np.float32(0.1)
    return v, i, (t, prm, pos, pool, poly), vel


@pytest.mark.parametrize("fix", [False, True])
@pytest.mark.parametrize("mesh_pose", [None, [0.0, 0.0, 0.0, 1.0, 0.25, -0.5, 0.125],
                                       [0.0, 0.2588190451, 0.0, 0.9659258263, 3.0, -0.25, -2.0]])
def test_trimesh_contacts_frames_bit_exact(gpu_ctx, oracle_lib, mesh_pose, fix):
    """With and without TriMeshFlags::FIX_INTERNAL_EDGES (normal constraints from pseudo-normals)."""
    O = oracle_lib
    v, i, (t, prm, pos, pool, poly), vel = _scene(300, 21)
    n = len(t)
    mesh = pg.TriMesh(gpu_ctx, v, i, flags=pg.TRIMESH_FIX_INTERNAL_EDGES if fix else 0)
    K = 256
    tc = pg.TriMeshContacts(gpu_ctx, mesh, n, K)
    ref = O.TriMeshContacts(v, i, n, fix_internal_edges=fix)
    mp = np.array([0, 0, 0, 1, 0, 0, 0], np.float32) if mesh_pose is None else np.array(mesh_pose, np.float32)
    moved = 0
    for f in range(6):
        pf = pos.copy()
        pf[:, 4:7] += vel * np.float32(f * (3 if f >= 4 else 1))
        s = ShapeSet.from_arrays(t, prm, pf, pool, poly)
        tc.update(s, 0.02, mesh_pose=None if mesh_pose is None else mp)
        ref.update(mp, s, 0.02)
        counts, tris, recs = tc.read()
        want_counts = np.array([len(x) for x in ref.inter], np.uint32)
        np.testing.assert_array_equal(counts, want_counts)
        assert counts.max() <= K and counts.sum() > 1000
        for sidx in range(n):
            c = counts[sidx]
            np.testing.assert_array_equal(tris[sidx, :c], ref.inter[sidx])
        got = np.concatenate([recs[sidx, :counts[sidx]] for sidx in range(n)])
        want = np.concatenate([ref.records[sidx].view(M.MANIFOLD_DTYPE).reshape(-1) for sidx in range(n)])
        got = got.copy()
        got["status"] = 0
        want = want.copy()
        want["status"] = 0
        assert_records_equal(got, want)
        if f == 0:
            first = [x.copy() for x in ref.inter]
        else:
            moved += sum(not np.array_equal(a, b) for a, b in zip(first, ref.inter))
    assert moved > 0
    assert (got["n_points"] > 0).sum() > 200
    tc.close()
    mesh.close()


def test_capacity_exceeded_is_reported(gpu_ctx):
    """More interfering triangles than the per-shape capacity raise CAPACITY_EXCEEDED (the list is
    truncated, never overrun); the context stays usable."""
    v, i, (t, prm, pos, pool, poly), vel = _scene(40, 5)
    n = len(t)
    mesh = pg.TriMesh(gpu_ctx, v, i)
    tc = pg.TriMeshContacts(gpu_ctx, mesh, n, 1)
    with pytest.raises(pg.ParryGpuError):
        tc.update(ShapeSet.from_arrays(t, prm, pos, pool, poly), 0.02)
    tc.close()
    tc = pg.TriMeshContacts(gpu_ctx, mesh, n, 256)
    tc.update(ShapeSet.from_arrays(t, prm, pos, pool, poly), 0.02)
    counts, _, _ = tc.read()
    assert counts.max() > 1
    tc.close()
    mesh.close()
