"""Triangle pseudo-normals and normal constraints (TriMeshFlags::FIX_INTERNAL_EDGES) in the oracle:
the reference's own projection tests (src/shape/triangle_pseudo_normals.rs:100-231, restated),
properties of the per-triangle tables, and the internal-edge fix on contact manifolds (CPU only)."""
import numpy as np
import pytest

from parry_gb300 import manifold as M
from parry_gb300 import workloads as W
from parry_gb300.shapes import ShapeSet, pose7

F = np.float32
Y = np.array([0, 1, 0], F)


def _normalize(v):
    v = np.asarray(v, F)
    n = np.sqrt(F(F(v[0] * v[0]) + F(v[1] * v[1])) + F(v[2] * v[2]))
    return (v / n).astype(F)


def _bisector(a, b):
    return _normalize(np.asarray(a, F) + np.asarray(b, F))


def _lerp(a, b, t):
    t = F(t)
    return (np.asarray(a, F) * (F(1) - t) + np.asarray(b, F) * t).astype(F)


def _pn(face, edges):
    return np.concatenate([np.asarray(face, F)] + [np.asarray(e, F) for e in edges]).reshape(1, 12)


def _project(O, pn, d):
    out, ok = O.project_local_normals(pn, np.asarray(d, F).reshape(1, 3))
    return out[0], bool(ok[0])


def flat_mesh(nx=8, nz=8, y=0.0):
    v, i = W.terrain_mesh(nx, nz)
    v = v.copy()
    v[:, 1] = y
    return v, i


def test_trivial_pseudo_normals_projection(oracle_lib):
    O = oracle_lib
    pn = _pn(Y, [Y, Y, Y])
    d, ok = _project(O, pn, [1, 1, 1])
    assert ok and np.array_equal(d, Y)
    _, ok = _project(O, pn, -Y)
    assert not ok


@pytest.mark.parametrize("negative", [False, True])
def test_edge_pseudo_normals_projection(oracle_lib, negative):
    O = oracle_lib
    ref = [np.array([0, 0, -1], F), np.array([-1, 0, 0], F), _normalize([1, 0, 1])]
    if negative:
        ends = [_bisector(r, -Y) for r in ref]
        axes = [_bisector(_bisector(r, Y), r) for r in ref]
    else:
        ends = [_bisector(r, Y) for r in ref]
        axes = [_bisector(e, Y) for e in ends]
    pn = _pn(Y, [_normalize(a) for a in axes])
    for i in range(3):
        d, ok = _project(O, pn, axes[i])
        assert ok and np.array_equal(d, axes[i])
        if not negative:
            d, ok = _project(O, pn, ends[i])
            assert ok and np.allclose(d, ends[i], atol=1e-5)
        for k in range(1, 100):
            v = _normalize(_lerp(Y, ends[i], k / 100))
            d, ok = _project(O, pn, v)
            assert ok and np.array_equal(d, v), (i, k)
        for k in range(1, 100):
            if negative:
                v = _normalize(_lerp(-Y, ends[i], k / 100))
                _, ok = _project(O, pn, v)
                assert not ok, (i, k)
            else:
                v = _normalize(_lerp(ref[i], ends[i], k / 100))
                d, ok = _project(O, pn, v)
                assert ok and np.allclose(d, ends[i], atol=1e-5), (i, k)
                v = _normalize(_lerp(ref[i], -Y, k / 100))
                _, ok = _project(O, pn, v)
                assert not ok, (i, k)


def test_flat_mesh_pseudo_normals_are_the_face_normal(oracle_lib):
    O = oracle_lib
    v, i = flat_mesh()
    pn, ok = O.trimesh_pseudo_normals(v, i)
    assert ok.all()
    assert np.array_equal(pn, np.tile(np.concatenate([Y] * 4), (len(i), 1)))


def test_duplicated_vertices_are_merged(oracle_lib):
    """FIX_INTERNAL_EDGES merges bit-identical vertices first: a triangle soup (three vertices of its
    own per triangle) gets the same constraints as the indexed mesh."""
    O = oracle_lib
    v, i = W.terrain_mesh(12, 9)
    soup_v = v[i].reshape(-1, 3)
    soup_i = np.arange(len(soup_v), dtype=np.uint32).reshape(-1, 3)
    a, oka = O.trimesh_pseudo_normals(v, i)
    b, okb = O.trimesh_pseudo_normals(soup_v, soup_i)
    assert oka.all() and np.array_equal(oka, okb)
    assert np.array_equal(a, b)
    # edge pseudo-normals of interior edges differ from the face normal on a bumpy terrain
    assert np.any(a[:, 3:6] != a[:, 0:3])


def test_folded_edge_has_no_constraints(oracle_lib):
    """Two triangles sharing an edge with opposite normals: that edge's pseudo-normal sums to zero,
    so neither triangle has constraints (triangle_normal_constraints returns None); a degenerate
    triangle has none either."""
    O = oracle_lib
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [0, 0, 0], [2, 0, 0], [3, 0, 0], [5, 0, 5]], F)
    i = np.array([[0, 2, 1], [0, 1, 2], [4, 5, 5], [0, 2, 6]], np.uint32)
    pn, ok = O.trimesh_pseudo_normals(v, i)
    assert not ok[0] and not ok[1] and not ok[2]
    assert ok[3]


def _grid_scene(n, seed, mesh):
    """Balls and cuboids resting on a mesh at y = 0 with a small penetration, spread over it."""
    v, i = mesh
    rng = np.random.default_rng(seed)
    s = ShapeSet()
    for k in range(n):
        x, z = rng.uniform(1.0, 7.0, 2)
        yaw = rng.uniform(0, np.pi)
        q = (0.0, np.sin(yaw / 2), 0.0, np.cos(yaw / 2))
        if k % 2 == 0:
            r = rng.uniform(0.2, 0.6)
            s.add_ball(r, pose7((x, r - 0.01, z)))
        else:
            he = rng.uniform(0.2, 0.7, 3)
            s.add_cuboid(tuple(he), pose7((x, he[1] - 0.01, z), q))
    return s


def _all_pairs_manifolds(O, mesh, shapes, fix, prediction=0.02):
    v, i = mesh
    tc = O.TriMeshContacts(v, i, len(shapes.arrays()[0]), fix_internal_edges=fix)
    tc.update(np.array([0, 0, 0, 1, 0, 0, 0], F), shapes, prediction, threads=1)
    recs = np.concatenate([r.view(M.MANIFOLD_DTYPE).reshape(-1) for r in tc.records])
    return recs


def test_internal_edges_fixed_on_a_flat_mesh(oracle_lib):
    """The internal-edge artefact and its fix: shapes resting on a flat tessellated plane get tilted
    normals from triangle edges they barely overlap; with FIX_INTERNAL_EDGES every generated
    manifold's normal is the plane normal."""
    O = oracle_lib
    mesh = flat_mesh()
    shapes = _grid_scene(40, 3, mesh)
    plain = _all_pairs_manifolds(O, mesh, shapes, False)
    fixed = _all_pairs_manifolds(O, mesh, shapes, True)
    live_p = plain[plain["n_points"] > 0]
    live_f = fixed[fixed["n_points"] > 0]
    assert len(live_p) > 40 and len(live_f) > 20
    assert np.any(np.abs(live_p["local_n1"] - Y).max(axis=1) > 1e-3)
    assert np.array_equal(live_f["local_n1"], np.tile(Y, (len(live_f), 1)))
    pts = np.concatenate([m["points"][: m["n_points"]] for m in live_f])
    assert np.all(pts["dist"] <= 0.02 + 1e-6)


def test_constraints_change_only_constrained_triangles(oracle_lib):
    """On a bumpy terrain, shapes far from any triangle edge of concern give the same manifolds
    with or without constraints where the GJK/SAT normal is already inside the cone; the fix is
    never a no-op over a whole scene."""
    O = oracle_lib
    v, i = W.terrain_mesh(24, 12, seed=5)
    t, prm, pos, pool, poly, _ = W.primitive_pairs(150, seed=6)
    rng = np.random.default_rng(1)
    pos = pos.copy()
    pos[:, 4] = rng.uniform(1, 23, len(t))
    pos[:, 6] = rng.uniform(1, 11, len(t))
    pos[:, 5] = rng.uniform(1.0, 4.0, len(t))
    s = ShapeSet.from_arrays(t, prm, pos, pool, poly)
    plain = _all_pairs_manifolds(O, (v, i), s, False)
    fixed = _all_pairs_manifolds(O, (v, i), s, True)
    assert len(plain) == len(fixed) and len(plain) > 500
    same = np.all(M.as_words(plain) == M.as_words(fixed), axis=1)
    assert same.mean() > 0.5 and not same.all()
