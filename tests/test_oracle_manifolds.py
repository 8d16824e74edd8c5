"""Contact manifolds: the oracle against the reference's doc-test known answers and geometric
properties (CPU only)."""
import json
from pathlib import Path

import numpy as np
import pytest

from parry_gb300 import manifold as M
from parry_gb300.shapes import ShapeSet, pose7, BALL, CUBOID, CAPSULE
from tests._contact_cases import primitive_scene, moved_poses
from tests._helpers import brute_force_pairs

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def _pair_scene(t1, p1, t2, p2, pos12_t, pos12_q=(0.0, 0.0, 0.0, 1.0)):
    """Shape 1 at the identity, shape 2 at pos12 (so the local frames are those of the reference call)."""
    s = ShapeSet.from_arrays(np.array([t1, t2], np.uint32), np.array([p1, p2], np.float32),
                             np.array([pose7(), pose7(pos12_t, pos12_q)], np.float32))
    return s


def _run(O, shapes, pairs, prediction, rec):
    st = O.contact_manifolds(shapes, np.asarray(pairs, np.uint32), prediction, M.as_words(rec), threads=1)
    return st


def test_ball_ball_doc_tests(oracle_lib):
    O = oracle_lib
    c = KA["manifold_ball_ball_overlap"]
    s = _pair_scene(BALL, (c["radius1"], 0, 0, 0), BALL, (c["radius2"], 0, 0, 0), c["pos12"])
    rec = M.new_manifolds(1)
    _run(O, s, [[0, 1]], c["prediction"], rec)
    m = rec[0]
    assert m["status"] == M.STATUS_OK and m["n_points"] == 1
    assert m["points"]["dist"][0] == pytest.approx(-0.5)
    np.testing.assert_array_equal(m["local_n1"], [1, 0, 0])
    np.testing.assert_array_equal(m["local_n2"], [-1, 0, 0])
    assert m["points"]["fid1"][0] == M.feature_face(0) and m["points"]["fid2"][0] == M.feature_face(0)

    c = KA["manifold_ball_ball_prediction"]
    s = _pair_scene(BALL, (c["radius1"], 0, 0, 0), BALL, (c["radius2"], 0, 0, 0), c["pos12"])
    rec = M.new_manifolds(1)
    _run(O, s, [[0, 1]], c["prediction"], rec)
    assert rec[0]["n_points"] == 1 and rec[0]["points"]["dist"][0] > 0.0
    # without prediction the separated balls have no contact
    rec = M.new_manifolds(1)
    _run(O, s, [[0, 1]], 0.0, rec)
    assert rec[0]["n_points"] == 0


def test_match_contacts_doc_test(oracle_lib):
    O = oracle_lib
    c = KA["manifold_match_contacts"]
    s1 = _pair_scene(BALL, (c["radius1"], 0, 0, 0), BALL, (c["radius2"], 0, 0, 0), c["pos12_frame1"])
    rec = M.new_manifolds(1)
    _run(O, s1, [[0, 1]], c["prediction"], rec)
    assert rec[0]["n_points"] == 1
    rec[0]["points"]["data"][0] = c["data"]
    s2 = _pair_scene(BALL, (c["radius1"], 0, 0, 0), BALL, (c["radius2"], 0, 0, 0), c["pos12_frame2"])
    _run(O, s2, [[0, 1]], c["prediction"], rec)
    assert rec[0]["n_points"] == 1
    assert rec[0]["points"]["data"][0] == c["data"]
    assert rec[0]["points"]["dist"][0] == pytest.approx(-0.15, abs=1e-6)


def test_cuboid_stack_doc_test(oracle_lib):
    O = oracle_lib
    c = KA["manifold_cuboid_stack"]
    s = _pair_scene(CUBOID, (*c["half_extents1"], 0), CUBOID, (*c["half_extents2"], 0), c["pos12"])
    rec = M.new_manifolds(1)
    _run(O, s, [[0, 1]], c["prediction"], rec)
    m = rec[0]
    n = int(m["n_points"])
    assert n >= 4
    np.testing.assert_array_equal(m["local_n1"], [0, 1, 0])
    np.testing.assert_array_equal(m["local_n2"], [0, -1, 0])
    pts = m["points"][:n]
    expect = np.float32(np.float32(1.9) - np.float32(2.0))
    np.testing.assert_allclose(pts["dist"], expect, atol=1e-6)
    # every point of shape 1 lies on its top face, inside the overlap square
    np.testing.assert_allclose(pts["local_p1"][:, 1], 1.0, atol=1e-6)
    assert np.all(np.abs(pts["local_p1"][:, [0, 2]]) <= 1.0 + 1e-6)
    # the four corners of the square are contact points
    corners = {(sx, sz) for sx in (-1.0, 1.0) for sz in (-1.0, 1.0)}
    got = {(float(np.round(p[0], 5)), float(np.round(p[2], 5))) for p in pts["local_p1"]}
    assert corners <= got
    d = M.find_deepest_contact(m)
    assert d is not None and pts["dist"][d] == pts["dist"].min()


def test_unsupported_pairs_leave_record(oracle_lib):
    """A convex vertex cloud without ConvexPolyhedron topology has no manifold generator: status
    Unsupported, record untouched; a triangle has one (the ball-triangle pair is generated)."""
    O = oracle_lib
    s = ShapeSet()
    s.add_ball(1.0)
    s.add_convex(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32), pose7((0.5, 0, 0)))
    s.add_triangle((0, 0, 0), (1, 0, 0), (0, 1, 0), pose7((0, 0.5, 0)))
    rec = M.new_manifolds(2)
    rec["n_points"] = 7
    rec["local_n1"] = 0.25
    before = rec.copy()
    st = O.contact_manifolds(s, np.array([[0, 1], [0, 2]], np.uint32), 0.1, M.as_words(rec), threads=1)
    assert st["unsupported"] == 1
    assert rec["status"][0] == M.STATUS_UNSUPPORTED and rec["status"][1] == M.STATUS_OK
    assert rec["n_points"][0] == before["n_points"][0]
    np.testing.assert_array_equal(rec["local_n1"][0], before["local_n1"][0])


def test_empty_slots_are_skipped(oracle_lib):
    """A pair row (PAIR_NONE, PAIR_NONE) is an empty slot: no query, record and status untouched,
    counted neither as a pair nor as unsupported."""
    O = oracle_lib
    s = ShapeSet()
    s.add_ball(1.0)
    s.add_ball(1.0, pose7((1.5, 0, 0)))
    rec = M.new_manifolds(3)
    rec["n_points"][1] = 9
    rec["status"][1] = 77
    pairs = np.array([[0, 1], [M.PAIR_NONE, M.PAIR_NONE], [1, 0]], np.uint32)
    st = O.contact_manifolds(s, pairs, 0.1, M.as_words(rec), threads=1)
    assert st["unsupported"] == 0
    assert rec["n_points"][1] == 9 and rec["status"][1] == 77
    assert rec["n_points"][0] == 1 and rec["n_points"][2] == 1


def _scene(n, seed, frame=0):
    t, p, q = primitive_scene(n, seed)
    if frame:
        q = moved_poses(q, frame, seed + 1)
    return ShapeSet.from_arrays(t, p, q)


def test_manifold_agrees_with_contact_query(oracle_lib):
    """The deepest manifold point and the contact query see the same pairs and depths."""
    O = oracle_lib
    shapes = _scene(600, 11)
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.1))
    assert len(pairs) > 300
    pred = 0.1
    rec = M.new_manifolds(len(pairs))
    st = O.contact_manifolds(shapes, pairs, pred, M.as_words(rec), threads=4)
    assert st["unsupported"] == 0 and st["max_points"] <= M.MAX_POINTS
    has, out, _ = O.contacts(shapes, pairs, pred, precision="f64", threads=4)
    n = rec["n_points"]
    # penetrating pairs have manifold points (separated pairs inside the prediction band may have
    # none: clipping of separated support features can come out empty, as in the reference)
    deep = has.astype(bool) & (out[:, 12] < -1e-3)
    assert np.all(n[deep] > 0)
    far = ~has.astype(bool)
    assert np.all(n[far] == 0)
    for k in np.nonzero(deep)[0]:
        d = M.find_deepest_contact(rec[k])
        # SAT / clipping and EPA find the same penetration depth up to f32 rounding
        assert rec[k]["points"]["dist"][d] == pytest.approx(out[k, 12], abs=2e-3), k


def test_frames_are_deterministic_and_carry_data(oracle_lib):
    """Frame-to-frame updates: same inputs give the same records; data follows feature ids."""
    O = oracle_lib
    n, seed, pred = 300, 5, 0.05
    pairs = brute_force_pairs(O.shape_aabbs(_scene(n, seed), 0.3))
    recs = [M.new_manifolds(len(pairs)), M.new_manifolds(len(pairs))]
    for f in range(4):
        shapes = _scene(n, seed, f)
        for r in recs:
            O.contact_manifolds(shapes, pairs, pred, M.as_words(r), threads=1 + 3 * (r is recs[1]))
        np.testing.assert_array_equal(M.as_words(recs[0]), M.as_words(recs[1]))
        # tag every live contact with its frame and index, as a solver would store impulses
        for r in recs:
            live = np.arange(M.MAX_POINTS)[None, :] < r["n_points"][:, None]
            r["points"]["data"] = np.where(live, f * 100 + np.arange(M.MAX_POINTS)[None, :], 0).astype(np.float32)
        prev = recs[0].copy()
        if f == 3:
            break
        shapes_next = _scene(n, seed, f + 1)
        O.contact_manifolds(shapes_next, pairs, pred, M.as_words(recs[0]), threads=1)
        carried = 0
        for k in range(len(pairs)):
            old = prev[k]["points"][:prev[k]["n_points"]]
            for c in recs[0][k]["points"][:recs[0][k]["n_points"]]:
                match = [o["data"] for o in old if o["fid1"] == c["fid1"] and o["fid2"] == c["fid2"]]
                if match:
                    assert c["data"] == match[-1]
                    carried += 1
        assert carried > 0
        recs[1] = recs[0].copy()
        recs[0] = prev.copy()
        O.contact_manifolds(shapes_next, pairs, pred, M.as_words(recs[0]), threads=4)
        np.testing.assert_array_equal(M.as_words(recs[0]), M.as_words(recs[1]))


def test_sliding_cuboid_stress(oracle_lib):
    """3-D counterpart of the reference's cuboids_large_size_ratio_issue_181 (a 2-D test): a cuboid
    pushed out of a long thin one along the manifold normal over many frames stays finite."""
    O = oracle_lib
    rec = M.new_manifolds(1)
    p = np.zeros(3)
    angle = 0.0
    for _ in range(2000):
        p[0] += 0.0001
        angle += 0.005
        q = (0.0, 0.0, np.sin(angle / 2), np.cos(angle / 2))
        # pos_ab = pos_a^-1 * pos_b with pos_b = translation (5, 0, 0) rotated 1.5 rad about z
        s = ShapeSet.from_arrays(np.array([CUBOID, CUBOID], np.uint32),
                                 np.array([[10, 10, 10, 0], [300, 1.5, 1.5, 0]], np.float32),
                                 np.array([pose7(p, q), pose7((5, 0, 0), (0, 0, np.sin(0.75), np.cos(0.75)))], np.float32))
        O.contact_manifolds(s, np.array([[0, 1]], np.uint32), 0.0, M.as_words(rec), threads=1)
        m = rec[0]
        assert np.all(np.isfinite(m["local_n1"]))
        d = M.find_deepest_contact(m)
        if d is not None:
            assert np.isfinite(m["points"]["dist"][d])
            n1w = _rotate(q, m["local_n1"].astype(np.float64))
            p += n1w * float(m["points"]["dist"][d])


def _rotate(q, v):
    x, y, z, w = q
    u = np.array([x, y, z])
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


@pytest.mark.parametrize("kinds", [(BALL, CUBOID), (CAPSULE, CUBOID), (CAPSULE, BALL)])
def test_flipped_pairs_mirror(oracle_lib, kinds):
    """(a, b) and (b, a) give mirrored manifolds for the analytic convex-ball path and agree on
    contact existence for the polygonal-feature path."""
    O = oracle_lib
    t, p, q = primitive_scene(400, 3)
    sel = np.isin(t, kinds)
    shapes = ShapeSet.from_arrays(t[sel], p[sel], q[sel])
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.0))
    tt = t[sel]
    pairs = pairs[tt[pairs[:, 0]] != tt[pairs[:, 1]]]
    assert len(pairs) > 5
    r1 = M.new_manifolds(len(pairs))
    r2 = M.new_manifolds(len(pairs))
    O.contact_manifolds(shapes, pairs, 0.0, M.as_words(r1), threads=1)
    O.contact_manifolds(shapes, pairs[:, ::-1].copy(), 0.0, M.as_words(r2), threads=1)
    np.testing.assert_array_equal(r1["n_points"] > 0, r2["n_points"] > 0)
    if BALL in kinds:
        live = r1["n_points"] > 0
        np.testing.assert_allclose(r1["points"]["dist"][live, 0], r2["points"]["dist"][live, 0], atol=2e-6)
        np.testing.assert_allclose(r1["points"]["local_p1"][live, 0], r2["points"]["local_p2"][live, 0], atol=2e-5)
        np.testing.assert_array_equal(r1["points"]["fid1"][live, 0], r2["points"]["fid2"][live, 0])


def test_hull_topology_is_a_convex_polyhedron():
    """The host hull builder's topology: closed (Euler V - E + F with merged faces), every vertex
    behind every face plane, unit normals, counter-clockwise faces, consistent adjacency."""
    from tests._contact_cases import hull_scene
    s, _ = hull_scene(64, 4)
    t, p, q, pool = s.arrays()
    hulls, topo = s.polyhedra()
    assert len(hulls) == 16 and np.all(hulls[:, 6] == 1)
    for r in hulls:
        v0, nv, f0, nf, e0, ne = (int(x) for x in r[:6])
        pts = pool[v0:v0 + nv].astype(np.float64)
        fr = topo["face_ranges"][f0:f0 + nf]
        fn = topo["face_normals"][f0:f0 + nf].astype(np.float64)
        np.testing.assert_allclose(np.linalg.norm(fn, axis=1), 1.0, atol=1e-6)
        assert int(fr[:, 1].sum()) >= 3 * nf and np.all(fr[:, 1] >= 3)
        for f in range(nf):
            vids = topo["face_vertices"][fr[f, 0]:fr[f, 0] + fr[f, 1]]
            a = pts[vids[0]]
            assert ((pts - a) @ fn[f]).max() < 1e-5
            # counter-clockwise around the outward normal
            c = np.cross(pts[vids[1]] - pts[vids[0]], pts[vids[2]] - pts[vids[0]])
            assert c @ fn[f] > 0
        # each vertex's adjacency lists the faces it belongs to
        vr = topo["vertex_ranges"][v0:v0 + nv]
        for v in range(nv):
            faces = set(topo["vertex_faces"][vr[v, 0]:vr[v, 0] + vr[v, 1]].tolist())
            expect = {f for f in range(nf) if v in topo["face_vertices"][fr[f, 0]:fr[f, 0] + fr[f, 1]]}
            assert faces == expect


def test_hull_manifolds_agree_with_contact_query(oracle_lib):
    """Hull pairs (pfm-pfm with ConvexPolyhedron features, convex-ball with hull features) against
    the contact query on the same scene."""
    from tests._contact_cases import hull_scene
    O = oracle_lib
    shapes, _ = hull_scene(700, 21)
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.1))
    t = shapes.arrays()[0]
    kinds = {(int(t[a]), int(t[b])) for a, b in pairs}
    assert {(3, 3), (0, 3), (1, 3), (2, 3)} & kinds
    pred = 0.1
    rec = M.new_manifolds(len(pairs))
    st = O.contact_manifolds(shapes, pairs, pred, M.as_words(rec), threads=4)
    assert st["unsupported"] == 0
    has, out, _ = O.contacts(shapes, pairs, pred, precision="f64", threads=4)
    n = rec["n_points"]
    deep = has.astype(bool) & (out[:, 12] < -1e-3)
    assert np.all(n[deep] > 0)
    assert np.all(n[~has.astype(bool)] == 0)
    hull_pairs = (t[pairs[:, 0]] == 3) | (t[pairs[:, 1]] == 3)
    checked = 0
    for k in np.nonzero(deep & hull_pairs)[0]:
        # the GJK/EPA point is one of the manifold points (pfm_pfm pushes it; convex-ball has only
        # it); clipped feature vertices may lie deeper along the normal
        dists = rec[k]["points"]["dist"][:n[k]]
        assert np.min(np.abs(dists - out[k, 12])) < 2e-3, k
        assert dists.min() <= out[k, 12] + 2e-3, k
        checked += 1
    assert checked > 50
    # hull-ball contacts carry the hull feature (face, edge or vertex) of the projection
    hb = np.nonzero(deep & (((t[pairs[:, 0]] == 3) & (t[pairs[:, 1]] == 0)) | ((t[pairs[:, 0]] == 0) & (t[pairs[:, 1]] == 3))))[0]
    assert len(hb) > 5
    for k in hb:
        f = rec[k]["points"]["fid1"][0] if t[pairs[k, 0]] == 3 else rec[k]["points"]["fid2"][0]
        assert (int(f) >> 30) in (1, 2, 3)


def test_init_dirs_seed_only_records_without_a_normal(oracle_lib):
    """init_dirs replaces the default GJK start (relative translation) only where a record holds no
    cached normal: zero rows are the plain call; once every record has a normal, any directions give
    the plain answer; on new records a start along the final direction shortens GJK and keeps the
    contact decision."""
    O = oracle_lib
    t, p, q0 = primitive_scene(800, 3, extent=5.0)
    shapes = ShapeSet.from_arrays(t, p, q0)
    pairs = brute_force_pairs(O.shape_aabbs(shapes, 0.3))
    ta, tb = t[pairs[:, 0]], t[pairs[:, 1]]
    poly = (ta != BALL) & (tb != BALL) & ~((ta == tb) & ((ta == CUBOID) | (ta == CAPSULE)))
    pairs = pairs[poly]
    assert len(pairs) > 200
    k = len(pairs)
    plain, zero = M.new_manifolds(k), M.new_manifolds(k)
    st_p = O.contact_manifolds(shapes, pairs, 0.05, M.as_words(plain))
    st_z = O.contact_manifolds(shapes, pairs, 0.05, M.as_words(zero), init_dirs=np.zeros((k, 3), np.float32))
    np.testing.assert_array_equal(M.as_words(plain), M.as_words(zero))
    assert st_p == st_z
    # warm records: a normal is cached for every pair with points, so random directions change nothing there
    has_n = np.linalg.norm(plain["local_n1"], axis=1) > 1e-3
    rng = np.random.default_rng(0)
    rnd = rng.normal(size=(k, 3)).astype(np.float32)
    moved = shapes.with_poses(moved_poses(q0, 1, 9, step=0.01, angle=0.01))
    a, b = plain.copy(), plain.copy()
    O.contact_manifolds(moved, pairs, 0.05, M.as_words(a))
    O.contact_manifolds(moved, pairs, 0.05, M.as_words(b), init_dirs=rnd)
    np.testing.assert_array_equal(M.as_words(a)[has_n], M.as_words(b)[has_n])
    # new records started along the plain run's final normal: the directions are used (the GJK runs
    # change) and the contact decisions are the plain ones
    sub = pairs[has_n]
    base, seeded = M.new_manifolds(len(sub)), M.new_manifolds(len(sub))
    st_b = O.contact_manifolds(shapes, sub, 0.05, M.as_words(base))
    st_s = O.contact_manifolds(shapes, sub, 0.05, M.as_words(seeded), init_dirs=np.ascontiguousarray(plain["local_n1"][has_n]))
    assert st_s["gjk_iters"] != st_b["gjk_iters"]
    np.testing.assert_array_equal(seeded["n_points"] > 0, base["n_points"] > 0)
    touching = base["n_points"] > 0  # (a pair beyond the prediction keeps whichever separating axis GJK stopped at)
    assert touching.sum() > 100
    np.testing.assert_allclose(seeded["local_n1"][touching], base["local_n1"][touching], atol=2e-3)
