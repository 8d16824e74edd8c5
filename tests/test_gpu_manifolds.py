"""Persistent contact manifolds on the GPU against the oracle: bit-exact records over several frames."""
import json
from pathlib import Path

import numpy as np
import pytest

from parry_gb300 import manifold as M
from parry_gb300.shapes import ShapeSet, pose7, BALL, CUBOID
from tests._contact_cases import primitive_scene, moved_poses
from tests._helpers import brute_force_pairs

pytestmark = pytest.mark.gpu

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def assert_records_equal(got: np.ndarray, want: np.ndarray):
    """Same status and point count; bit-identical normals and valid points."""
    np.testing.assert_array_equal(got["status"], want["status"])
    np.testing.assert_array_equal(got["n_points"], want["n_points"])
    gw, ww = M.as_words(got), M.as_words(want)
    np.testing.assert_array_equal(gw[:, 2:8], ww[:, 2:8])
    n = want["n_points"].astype(np.int64)
    valid = np.arange(M.MAX_POINTS)[None, :] < n[:, None]
    gp = gw[:, 8:].reshape(len(got), M.MAX_POINTS, 10)
    wp = ww[:, 8:].reshape(len(want), M.MAX_POINTS, 10)
    bad = np.nonzero(np.any(gp[valid] != wp[valid], axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} points differ"


def _both(O, pg, ctx, shapes, pairs, pred, rec_gpu, rec_cpu):
    pg.contact_manifolds(ctx, shapes, pairs, pred, rec_gpu)
    O.contact_manifolds(shapes, pairs, pred, M.as_words(rec_cpu))


def test_doc_test_cases(gpu_ctx, oracle_lib):
    import parry_gb300 as pg
    O = oracle_lib
    for key in ("manifold_ball_ball_overlap", "manifold_ball_ball_prediction"):
        c = KA[key]
        s = ShapeSet.from_arrays(np.array([BALL, BALL], np.uint32), np.array([[c["radius1"], 0, 0, 0], [c["radius2"], 0, 0, 0]], np.float32),
                                 np.array([pose7(), pose7(c["pos12"])], np.float32))
        g, w = M.new_manifolds(1), M.new_manifolds(1)
        _both(O, pg, gpu_ctx, s, np.array([[0, 1]], np.uint32), c["prediction"], g, w)
        assert g["n_points"][0] == 1
        assert_records_equal(g, w)
    c = KA["manifold_cuboid_stack"]
    s = ShapeSet.from_arrays(np.array([CUBOID, CUBOID], np.uint32),
                             np.array([[*c["half_extents1"], 0], [*c["half_extents2"], 0]], np.float32),
                             np.array([pose7(), pose7(c["pos12"])], np.float32))
    g, w = M.new_manifolds(1), M.new_manifolds(1)
    _both(O, pg, gpu_ctx, s, np.array([[0, 1]], np.uint32), c["prediction"], g, w)
    assert g["n_points"][0] >= 4
    assert_records_equal(g, w)


@pytest.mark.parametrize("seed", [1, 2])
def test_frames_bit_exact(gpu_ctx, oracle_lib, seed):
    """Several frames of a drifting scene: every pair kind, warm records, data carried by feature ids."""
    import parry_gb300 as pg
    O = oracle_lib
    t, p, q0 = primitive_scene(1500, seed, extent=6.0)
    pred = 0.05
    pairs = brute_force_pairs(O.shape_aabbs(ShapeSet.from_arrays(t, p, q0), 0.4))
    assert len(pairs) > 2000
    kinds = {(int(t[a]), int(t[b])) for a, b in pairs}
    assert len(kinds) >= 8
    g, w = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    for f in range(5):
        shapes = ShapeSet.from_arrays(t, p, moved_poses(q0, f, seed + 100, step=0.02, angle=0.02))
        _both(O, pg, gpu_ctx, shapes, pairs, pred, g, w)
        assert_records_equal(g, w)
        assert np.all(g["status"] == M.STATUS_OK)
        # a solver would store impulses in `data`; give both the same values
        vals = (np.arange(len(pairs) * M.MAX_POINTS, dtype=np.float32).reshape(-1, M.MAX_POINTS) + f * 0.5)
        g["points"]["data"] = vals
        w["points"]["data"] = vals
    assert int(g["n_points"].sum()) > len(pairs) // 4


def test_device_records_in_place(gpu_ctx, oracle_lib):
    """Records resident in device memory (a CUDA tensor) are updated in place, as host records are."""
    torch = pytest.importorskip("torch")
    import parry_gb300 as pg
    O = oracle_lib
    t, p, q = primitive_scene(800, 9, extent=5.0)
    shapes = ShapeSet.from_arrays(t, p, q)
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.2))
    w = M.new_manifolds(len(pairs))
    d = torch.zeros((len(pairs), M.RECORD_WORDS), dtype=torch.int32, device="cuda")
    tt, pp, qq, pool = shapes.arrays()
    dev_shapes = (torch.from_numpy(tt.view(np.int32)).cuda(), torch.from_numpy(pp).cuda(), torch.from_numpy(qq).cuda(),
                  torch.from_numpy(pool).cuda())
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    for f in range(3):
        q2 = moved_poses(q, f, 77)
        dev_shapes = (dev_shapes[0], dev_shapes[1], torch.from_numpy(q2).cuda(), dev_shapes[3])
        pg.contact_manifolds(gpu_ctx, dev_shapes, dpairs, 0.02, d)
        gpu_ctx.sync()
        O.contact_manifolds(ShapeSet.from_arrays(t, p, q2), pairs, 0.02, M.as_words(w))
        got = M.as_records(d.cpu().numpy().view(np.uint32).copy())
        assert_records_equal(got, w)


def test_unsupported_and_invalid(gpu_ctx, oracle_lib):
    import parry_gb300 as pg
    O = oracle_lib
    s = ShapeSet()
    s.add_ball(1.0)
    s.add_convex(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32), pose7((0.5, 0, 0)))
    s.add_cuboid((1, 1, 1), pose7((0, 1.5, 0)))
    pairs = np.array([[0, 1], [0, 2]], np.uint32)
    g, w = M.new_manifolds(2), M.new_manifolds(2)
    g["n_points"][0] = 3
    w["n_points"][0] = 3
    _both(O, pg, gpu_ctx, s, pairs, 0.0, g, w)
    assert g["status"][0] == M.STATUS_UNSUPPORTED and g["n_points"][0] == 3
    assert g["status"][1] == M.STATUS_OK and g["n_points"][1] == 1
    assert_records_equal(g, w)
    bad = np.array([[0, 7]], np.uint32)
    r = M.new_manifolds(1)
    with pytest.raises(pg.ParryGpuError):
        pg.contact_manifolds(gpu_ctx, s, bad, 0.0, r)
    assert r["status"][0] == 1  # PARRYGPU_INVALID_ARG


def test_empty_slots_skipped(gpu_ctx, oracle_lib):
    """Rows (PAIR_NONE, PAIR_NONE) of a fixed-capacity pair list are skipped: their records (status
    included) stay as they were, the other rows match the oracle."""
    import parry_gb300 as pg
    O = oracle_lib
    t, p, q = primitive_scene(400, 5, extent=4.0)
    shapes = ShapeSet.from_arrays(t, p, q)
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.2)).copy()
    assert len(pairs) > 20
    empty = np.arange(0, len(pairs), 3)
    pairs[empty] = M.PAIR_NONE
    g, w = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    for r in (g, w):
        r["n_points"][empty] = 5
        r["status"][empty] = 77
    _both(O, pg, gpu_ctx, shapes, pairs, 0.02, g, w)
    assert np.all(g["n_points"][empty] == 5) and np.all(g["status"][empty] == 77)
    assert_records_equal(g, w)
    assert (g["n_points"] > 0).sum() > len(empty)


@pytest.mark.parametrize("seed", [3, 4])
def test_hull_frames_bit_exact(gpu_ctx, oracle_lib, seed):
    """Scenes with ConvexPolyhedron hulls (16-64 points) next to balls, cuboids and capsules, over
    several frames: pfm-pfm with hull faces, convex-ball with hull features, EPA fallbacks."""
    import parry_gb300 as pg
    from tests._contact_cases import hull_scene
    O = oracle_lib
    shapes0, q0 = hull_scene(1600, seed, extent=6.0)
    pairs = brute_force_pairs(O.shape_aabbs(shapes0, 0.3))
    t = shapes0.arrays()[0]
    kinds = {(int(t[a]), int(t[b])) for a, b in pairs}
    assert {(3, 3), (0, 3), (1, 3), (2, 3)} <= kinds or {(3, 3), (3, 0), (3, 1), (3, 2)} & kinds
    g, w = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    for f in range(4):
        shapes = shapes0.with_poses(moved_poses(q0, f, seed + 200, step=0.02, angle=0.02))
        st = pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, g, want_stats=True)
        O.contact_manifolds(shapes, pairs, 0.05, M.as_words(w))
        assert_records_equal(g, w)
        assert np.all(g["status"] == M.STATUS_OK)
        if f == 0:
            assert st["epa_calls"] > 0
        vals = np.arange(len(pairs) * M.MAX_POINTS, dtype=np.float32).reshape(-1, M.MAX_POINTS) * 0.25 + f
        g["points"]["data"] = vals
        w["points"]["data"] = vals


def test_triangle_pairs_frames_bit_exact(gpu_ctx, oracle_lib):
    """Triangles of a height field (as Triangle shapes at the mesh pose) against balls, cuboids,
    capsules and hulls settling onto them, over several frames: convex-ball with triangle
    features, cuboid-triangle SAT, polyhedral pairs with the triangle face."""
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    O = oracle_lib
    v, i = W.terrain_mesh(48, 24, seed=13)
    t, prm, pos, pool, poly, _ = W.primitive_pairs(300, seed=17)
    n = len(t)
    rng = np.random.default_rng(17)
    pos = pos.copy()
    pos[:, 4] = rng.uniform(1, 47, n)
    pos[:, 6] = rng.uniform(1, 23, n)
    pos[:, 5] = rng.uniform(0.5, 5.0, n)
    mesh_pose = np.array([0.0, 0.0, 0.0, 1.0, 0.3, -0.2, 0.1], np.float32)
    tri = np.ascontiguousarray(v[i], np.float32)
    shapes = O._with_triangles(ShapeSet.from_arrays(t, prm, pos, pool, poly), tri, mesh_pose)
    aabbs = O.shape_aabbs(shapes, 0.05)
    a_s, a_t = aabbs[:n], aabbs[n:]
    hit = np.all(a_s[:, None, :3] <= a_t[None, :, 3:], 2) & np.all(a_s[:, None, 3:] >= a_t[None, :, :3], 2)
    si, ti = np.nonzero(hit)
    pairs = np.stack([ti + n, si], 1).astype(np.uint32)
    kinds = {int(t[s]) for s in si}
    assert kinds == {0, 1, 2, 3} and len(pairs) > 2000
    g, w = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    for f in range(4):
        pf = pos.copy()
        pf[:, 5] -= 0.08 * f
        fs = O._with_triangles(ShapeSet.from_arrays(t, prm, pf, pool, poly), tri, mesh_pose)
        pg.contact_manifolds(gpu_ctx, fs, pairs, 0.05, g)
        O.contact_manifolds(fs, pairs, 0.05, M.as_words(w))
        assert_records_equal(g, w)
        assert np.all(g["status"] == M.STATUS_OK)
        assert (g["n_points"] > 0).sum() > 200


def test_with_dirs_bit_exact(gpu_ctx, oracle_lib):
    """parrygpu_contact_manifolds_with_dirs against the oracle given the same directions, over frames
    of a hull scene: unit directions, zero rows and NaN rows (neither normalises: the default start
    stays). Pairs with a cached normal ignore their direction, so later frames use it only for the
    pairs whose last update left no normal."""
    import parry_gb300 as pg
    from tests._contact_cases import hull_scene
    O = oracle_lib
    shapes0, q0 = hull_scene(1600, 5, extent=6.0)
    pairs = brute_force_pairs(O.shape_aabbs(shapes0, 0.3))
    rng = np.random.default_rng(5)
    dirs = rng.normal(size=(len(pairs), 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dirs[::7] = 0.0
    dirs[3::11] = np.nan
    g, w, plain = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    for f in range(3):
        shapes = shapes0.with_poses(moved_poses(q0, f, 305, step=0.02, angle=0.02))
        st = pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, g, want_stats=True, init_dirs=dirs)
        sto = O.contact_manifolds(shapes, pairs, 0.05, M.as_words(w), init_dirs=dirs)
        assert_records_equal(g, w)
        assert np.all(g["status"] == M.STATUS_OK)
        assert (st["gjk_iters"], st["epa_iters"], st["epa_calls"]) == (sto["gjk_iters"], sto["epa_iters"], sto["epa_calls"])
        stp = pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, plain, want_stats=True)
        if f == 0:  # every record is new: the random starts change the GJK runs
            assert stp["gjk_iters"] != st["gjk_iters"]
    # zero directions everywhere are the plain call
    z, p2 = M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))
    pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, z, init_dirs=np.zeros((len(pairs), 3), np.float32))
    pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, p2)
    assert_records_equal(z, p2)


def test_pipelined_host_records_match_device_records(gpu_ctx):
    """A large batch with host records runs in chunks (uploads, kernels and downloads overlapped on
    three streams): its records equal those of the same update on device records, frame after frame."""
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    t, prm, pos0, pool, poly, pairs = W.primitive_pairs(600_000)
    k = len(pairs)
    host = M.new_manifolds(k)
    dev = torch.zeros((k, M.RECORD_WORDS), dtype=torch.int32, device="cuda")
    for f in range(3):
        shapes = ShapeSet.from_arrays(t, prm, W.drifted_poses(pos0, f), pool, poly)
        pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, host)
        pg.contact_manifolds(gpu_ctx, shapes, pairs, 0.05, dev)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(M.as_words(host), dev.cpu().numpy().view(np.uint32))
    assert int((host["n_points"] > 0).sum()) > k // 10
