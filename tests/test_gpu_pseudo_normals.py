"""Triangle pseudo-normals (TriMeshFlags::FIX_INTERNAL_EDGES) on the GPU against the oracle: the
per-triangle constraint tables bit for bit (merged vertices, non-manifold and folded edges,
degenerate triangles), the projection of directions into the normal cones (the reference's own
projection tests restated, then random rows bit for bit), and the internal-edge fix on manifolds
against a flat tessellated plane."""
import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import manifold as M
from parry_gb300 import workloads as W
from parry_gb300.shapes import ShapeSet
from tests.test_oracle_pseudo_normals import (F, Y, _bisector, _lerp, _normalize, _pn, _grid_scene, flat_mesh)

pytestmark = pytest.mark.gpu


def _tables(ctx, O, v, i):
    mesh = pg.TriMesh(ctx, v, i, flags=pg.TRIMESH_FIX_INTERNAL_EDGES)
    got, gok = mesh.normal_constraints()
    mesh.close()
    want, wok = O.trimesh_pseudo_normals(v, i)
    return got, gok, want, wok


def _meshes():
    v, i = W.terrain_mesh()
    yield "terrain", v, i
    sv, si = W.terrain_mesh(40, 30, seed=3)
    yield "soup", sv[si].reshape(-1, 3).copy(), np.arange(3 * len(si), dtype=np.uint32).reshape(-1, 3)
    yield "flat", *flat_mesh(16, 16)
    # folded edge, a degenerate triangle, a non-manifold edge shared by three triangles, repeated
    # vertex positions under different indices
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [0, 0, 0], [2, 0, 0], [3, 0, 0], [5, 0, 5], [0, 1, 0], [0, -1, 0.5],
                  [1, 0, 0]], F)
    i = np.array([[0, 2, 1], [0, 1, 2], [4, 5, 5], [0, 2, 6], [3, 9, 7], [0, 1, 8], [7, 8, 9]], np.uint32)
    yield "odd", v, i


@pytest.mark.parametrize("case", ["terrain", "soup", "flat", "odd"])
def test_pseudo_normal_tables_bit_exact(gpu_ctx, oracle_lib, case):
    name, v, i = next(m for m in _meshes() if m[0] == case)
    got, gok, want, wok = _tables(gpu_ctx, oracle_lib, v, i)
    np.testing.assert_array_equal(gok, wok)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    if case != "odd":
        assert wok.all()


def test_flags_without_fix_give_no_constraints(gpu_ctx):
    v, i = flat_mesh(4, 4)
    mesh = pg.TriMesh(gpu_ctx, v, i, flags=pg.TRIMESH_ORIENTED)
    pn, ok = mesh.normal_constraints()
    assert not ok.any() and not pn.any()
    mesh.set_flags(pg.TRIMESH_FIX_INTERNAL_EDGES)
    assert mesh.normal_constraints()[1].all()
    mesh.set_flags(0)
    assert not mesh.normal_constraints()[1].any()
    with pytest.raises(pg.ParryGpuError):
        mesh.set_flags(1)  # HALF_EDGE_TOPOLOGY is not supported


def test_projection_reference_cases(gpu_ctx, oracle_lib):
    """triangle_pseudo_normals.rs:115-231 on the GPU: the same answers as the oracle, bit for bit."""
    ref = [np.array([0, 0, -1], F), np.array([-1, 0, 0], F), _normalize([1, 0, 1])]
    rows, dirs = [], []
    for negative in (False, True):
        if negative:
            ends = [_bisector(r, -Y) for r in ref]
            axes = [_bisector(_bisector(r, Y), r) for r in ref]
        else:
            ends = [_bisector(r, Y) for r in ref]
            axes = [_bisector(e, Y) for e in ends]
        pn = _pn(Y, [_normalize(a) for a in axes])
        for k in range(3):
            cand = [axes[k], ends[k]]
            for s in range(1, 100):
                cand.append(_normalize(_lerp(Y, ends[k], s / 100)))
                cand.append(_normalize(_lerp(ref[k], ends[k], s / 100)))
                cand.append(_normalize(_lerp(ref[k], -Y, s / 100)))
                cand.append(_normalize(_lerp(-Y, ends[k], s / 100)))
            rows += [pn[0]] * len(cand)
            dirs += cand
    rows.append(_pn(Y, [Y, Y, Y])[0])
    dirs.append(np.array([1, 1, 1], F))
    rows.append(_pn(Y, [Y, Y, Y])[0])
    dirs.append(-Y)
    rows, dirs = np.array(rows, F), np.array(dirs, F)
    got, gok = pg.project_local_normals(gpu_ctx, rows, dirs)
    want, wok = oracle_lib.project_local_normals(rows, dirs)
    np.testing.assert_array_equal(gok, wok)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(got[-2], Y) and gok[-2] and not gok[-1]


def test_projection_random_rows_bit_exact(gpu_ctx, oracle_lib):
    v, i = W.terrain_mesh(64, 32, seed=9)
    pn, ok = oracle_lib.trimesh_pseudo_normals(v, i)
    rng = np.random.default_rng(4)
    rows = pn[ok][rng.integers(0, ok.sum(), 200000)]
    d = rng.normal(size=(len(rows), 3)).astype(F)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(F)
    # half of the directions near each row's face normal, where the cone test decides
    d[::2] = rows[::2, :3] + F(0.3) * d[::2]
    got, gok = pg.project_local_normals(gpu_ctx, rows, d)
    want, wok = oracle_lib.project_local_normals(rows, d)
    np.testing.assert_array_equal(gok, wok)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    changed = np.any(got != d, axis=1)
    assert 0.05 < changed.mean() < 0.95 and 0.05 < (~gok).mean() < 0.95


def test_internal_edges_fixed_on_gpu(gpu_ctx, oracle_lib):
    """Shapes resting on a flat tessellated plane: with FIX_INTERNAL_EDGES every manifold normal is
    the plane normal on the GPU, and the records equal the oracle's."""
    v, i = flat_mesh()
    shapes = _grid_scene(40, 3, (v, i))
    n = len(shapes.arrays()[0])
    mesh = pg.TriMesh(gpu_ctx, v, i, flags=pg.TRIMESH_FIX_INTERNAL_EDGES)
    tc = pg.TriMeshContacts(gpu_ctx, mesh, n, 64)
    tc.update(shapes, 0.02)
    counts, tris, recs = tc.read()
    ref = oracle_lib.TriMeshContacts(v, i, n, fix_internal_edges=True)
    ref.update(np.array([0, 0, 0, 1, 0, 0, 0], F), shapes, 0.02)
    got = np.concatenate([recs[s, :counts[s]] for s in range(n)])
    want = np.concatenate([ref.records[s].view(M.MANIFOLD_DTYPE).reshape(-1) for s in range(n)])
    live = got[got["n_points"] > 0]
    assert len(live) > 20
    assert np.array_equal(live["local_n1"], np.tile(Y, (len(live), 1)))
    from tests.test_gpu_manifolds import assert_records_equal
    got, want = got.copy(), want.copy()
    got["status"] = 0
    want["status"] = 0
    assert_records_equal(got, want)
    tc.close()
