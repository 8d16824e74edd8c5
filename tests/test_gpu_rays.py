"""Parity of the CUDA ray-cast path (through the C ABI) with the oracle's f32 restatement of
parry3d: hit triangle / face ids identical, toi and normals within 1e-5 relative (f32 rounding of
the same arithmetic; observed differences are 0), and the error against the f64 oracle stated."""
import json
from pathlib import Path

import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import workloads as W

pytestmark = pytest.mark.gpu
REL = 1e-5
KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def _compare(f, t, n, fo, to, no):
    np.testing.assert_array_equal(f, fo)
    hit = fo != pg.NO_HIT
    np.testing.assert_allclose(t[hit], to[hit], rtol=REL, atol=0)
    np.testing.assert_allclose(n[hit], no[hit], rtol=REL, atol=REL)


def test_known_answers(gpu_ctx):
    case = KA["trimesh_culling_triangle"]
    m = pg.TriMesh(gpu_ctx, np.array(case["vertices"], np.float32), np.array(case["indices"], np.uint32))
    rays = np.array([r["origin"] + r["dir"] for r in case["rays"]], np.float32)
    f, t, n = m.cast_rays_and_get_normal(rays, case["max_toi"])
    for k, r in enumerate(case["rays"]):
        assert f[k] == r["expect_feature"]
        assert t[k] == pytest.approx(r["expect_toi"], rel=1e-6)
        np.testing.assert_allclose(n[k], r["expect_normal"], atol=1e-6)


def test_golden_fixture(gpu_ctx):
    g = np.load(Path(__file__).parent / "golden" / "terrain_small.npz")
    m = pg.TriMesh(gpu_ctx, g["vertices"], g["indices"])
    f, t, n = m.cast_rays_and_get_normal(g["rays"], float(g["max_toi"]))
    _compare(f, t, n, g["feature_f32"], g["toi_f32"], g["normal_f32"])


@pytest.mark.parametrize("sort_rays,key,traversal,refill", [(True, 0, 1, 0), (True, 1, 1, 0), (True, 2, 1, 0), (False, 0, 1, 0),
                                                        (False, 0, 2, 8), (True, 0, 2, 16), (False, 0, 2, 32), (True, 2, 2, 1),
                                                        (False, 0, 3, 0), (True, 1, 3, 0)])
def test_medium_terrain_vs_oracle(oracle_lib, sort_rays, key, traversal, refill):
    ctx = pg.Context(0, sort_rays=sort_rays, ray_sort_key=key, ray_traversal=traversal, ray_refill=refill)
    v, i = W.terrain_mesh(64, 32, seed=21)
    rays = W.terrain_rays(200_000, 64, 32, seed=21)
    m = pg.TriMesh(ctx, v, i)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0)
    _compare(f, t, n, fo, to, no)
    ctx.close()


def test_full_size_terrain_vs_oracle(gpu_ctx, oracle_lib):
    """The 65,536-triangle terrain and 1,048,576 rays: identical hit sets; error vs f64 stated."""
    v, i = W.terrain_mesh()
    rays = W.terrain_rays(1 << 20)
    m = pg.TriMesh(gpu_ctx, v, i)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)
    om = oracle_lib.TriMesh(v, i)
    fo, to, no = om.cast_rays_and_get_normal(rays, 100.0)
    _compare(f, t, n, fo, to, no)
    f64, t64, _ = oracle_lib.TriMesh(v, i, "f64").cast_rays_and_get_normal(rays, 100.0)
    hit = (fo != pg.NO_HIT) & (f64 == fo)
    err = np.abs(t[hit].astype(np.float64) - t64[hit]) / np.abs(t64[hit])
    print(f"\ntoi rel err vs f64 oracle: max {err.max():.3e} p99 {np.quantile(err, 0.99):.3e}; "
          f"feature mismatches vs f64: {(f64 != fo).sum()}")
    assert err.max() < 1e-4


def test_pose_and_cast_ray_variant(gpu_ctx, oracle_lib):
    v, i = W.terrain_mesh(32, 16, seed=4)
    rays = W.terrain_rays(50_000, 32, 16, seed=4)
    q = np.array([0.1, 0.2, -0.3, 0.9], np.float64)
    q /= np.linalg.norm(q)
    pose = np.array(list(q) + [3.0, -2.0, 1.5], np.float32)
    # move rays into the posed frame roughly: rotate is irrelevant for parity; just use them
    m = pg.TriMesh(gpu_ctx, v, i)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0, pose=pose)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0, pose=pose)
    _compare(f, t, n, fo, to, no)
    f2, t2 = m.cast_rays(rays, 100.0, pose=pose)
    np.testing.assert_array_equal(f2, f)
    np.testing.assert_array_equal(t2, t)


@pytest.mark.parametrize("traversal", [2, 3])
def test_fetch_traversal_full_size_pose_and_no_normal(oracle_lib, traversal):
    """The persistent dynamic-fetch and the postponed-leaf traversals on the full terrain workload,
    with a mesh pose, and through the toi-only variant, answer as the oracle."""
    ctx = pg.Context(0, ray_traversal=traversal)
    v, i = W.terrain_mesh()
    rays = W.terrain_rays(1 << 20, seed=77)
    m = pg.TriMesh(ctx, v, i)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)
    om = oracle_lib.TriMesh(v, i)
    fo, to, no = om.cast_rays_and_get_normal(rays, 100.0)
    _compare(f, t, n, fo, to, no)
    q = np.array([0.05, -0.1, 0.02, 0.99], np.float64)
    q /= np.linalg.norm(q)
    pose = np.array(list(q) + [1.0, 0.5, -2.0], np.float32)
    sub = rays[:200_000]
    f, t, n = m.cast_rays_and_get_normal(sub, 100.0, pose=pose)
    fo, to, no = om.cast_rays_and_get_normal(sub, 100.0, pose=pose)
    _compare(f, t, n, fo, to, no)
    f2, t2 = m.cast_rays(sub, 100.0, pose=pose)
    np.testing.assert_array_equal(f2, f)
    np.testing.assert_array_equal(t2, t)
    ctx.close()


def test_device_and_pinned_buffers(gpu_ctx, oracle_lib):
    import torch
    v, i = W.terrain_mesh(32, 16, seed=8)
    rays = W.terrain_rays(100_000, 32, 16, seed=8)
    m = pg.TriMesh(gpu_ctx, torch.from_numpy(v).cuda(), torch.from_numpy(i.view(np.int32)).cuda())
    fd, td, nd = m.cast_rays_and_get_normal(torch.from_numpy(rays).cuda(), 100.0)
    gpu_ctx.sync()
    fp, tp, np_ = m.cast_rays_and_get_normal(torch.from_numpy(rays).pin_memory(), 100.0)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0)
    _compare(fd.cpu().numpy().view(np.uint32), td.cpu().numpy(), nd.cpu().numpy(), fo, to, no)
    _compare(fp.numpy().view(np.uint32), tp.numpy(), np_.numpy(), fo, to, no)


def test_edge_cases(gpu_ctx):
    # empty mesh: every ray misses
    m0 = pg.TriMesh(gpu_ctx, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    f, t, n = m0.cast_rays_and_get_normal(np.array([[0, 1, 0, 0, -1, 0]], np.float32), 10.0)
    assert f[0] == pg.NO_HIT
    # zero rays
    m1 = pg.TriMesh(gpu_ctx, np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32), np.array([[0, 2, 1]], np.uint32))
    f, t, n = m1.cast_rays_and_get_normal(np.zeros((0, 6), np.float32), 10.0)
    assert len(f) == 0
    # single triangle (partial root), hit exactly at max_toi is rejected (strict <)
    r = np.array([[0.2, 1, 0.2, 0, -1, 0], [0.2, 2, 0.2, 0, -1, 0]], np.float32)
    f, t, n = m1.cast_rays_and_get_normal(r, 2.0)
    assert f[0] == 0 and t[0] == pytest.approx(1.0)
    assert f[1] == pg.NO_HIT
    # out-of-range index is rejected
    with pytest.raises(pg.ParryGpuError):
        pg.TriMesh(gpu_ctx, np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.uint32))


def test_autotune_keeps_answers(oracle_lib):
    """The autotuner picks one of its candidates, installs it in the context, and the answers
    after tuning are the oracle's."""
    ctx = pg.Context(0)
    v, i = W.terrain_mesh(64, 32, seed=5)
    rays = W.terrain_rays(100_000, 64, 32, seed=5)
    m = pg.TriMesh(ctx, v, i)
    cfg = m.autotune(rays, 100.0, reps=1)
    assert cfg["ray_sort_key"] in (0, 1, 2) and cfg["ray_traversal"] in (1, 2, 3)
    if cfg["ray_traversal"] in (1, 3):
        assert cfg["ray_block"] in (64, 128, 256)
    else:
        assert cfg["ray_refill"] in (8, 16, 24)
    assert ctx.config == cfg
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0)
    _compare(f, t, n, fo, to, no)
    ctx.close()


@pytest.mark.parametrize("kw", [{"ray_block": 48}, {"ray_block": 2048}, {"ray_sort_key": 3}, {"epa_blocks_per_sm": 64},
                                {"ray_traversal": 4}, {"ray_refill": 33}, {"ray_chunks": 65}])
def test_invalid_config_rejected(kw):
    with pytest.raises(Exception):
        pg.Context(0, **kw)


@pytest.mark.parametrize("traversal,chunks", [(1, 0), (2, 0), (3, 0), (1, 1), (1, 3), (1, 64)])
def test_pipelined_host_buffers(oracle_lib, traversal, chunks):
    """Host-buffer calls without a ray ordering, staged (ray_host_access = 2), run in chunks over two
    streams; pageable, pinned, device-in / host-out and toi-only calls all answer as the oracle."""
    import torch
    ctx = pg.Context(0, sort_rays=False, ray_traversal=traversal, ray_chunks=chunks, ray_host_access=2)
    v, i = W.terrain_mesh(128, 64, seed=9)
    rays = W.terrain_rays(600_001, 128, 64, seed=9)  # not a multiple of the chunk size
    m = pg.TriMesh(ctx, v, i)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)  # pageable numpy
    _compare(f, t, n, fo, to, no)
    fp, tp, np_ = m.cast_rays_and_get_normal(torch.from_numpy(rays).pin_memory(), 100.0)  # pinned
    _compare(fp.numpy().view(np.uint32), tp.numpy(), np_.numpy(), fo, to, no)
    feat = np.empty(len(rays), np.uint32)
    toi = np.empty(len(rays), np.float32)
    m.cast_rays(torch.from_numpy(rays).cuda(), 100.0, out=(feat, toi, None))  # device in, host out, no normals
    np.testing.assert_array_equal(feat, fo)
    np.testing.assert_array_equal(toi, t)
    ctx.close()


@pytest.mark.parametrize("traversal", [1, 2, 3])
def test_in_place_host_access(oracle_lib, traversal):
    """ray_host_access = 1: with page-locked host buffers the traversal reads the rays and writes
    the results in place (no staging); pageable buffers still go through the staged path. Answers
    equal the oracle's either way."""
    import torch
    ctx = pg.Context(0, sort_rays=False, ray_traversal=traversal, ray_host_access=1)
    assert ctx.config["ray_host_access"] == 1
    v, i = W.terrain_mesh(128, 64, seed=9)
    rays = W.terrain_rays(300_001, 128, 64, seed=9)
    m = pg.TriMesh(ctx, v, i)
    fo, to, no = oracle_lib.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0)
    rp = torch.from_numpy(rays).pin_memory()
    fp = torch.empty(len(rays), dtype=torch.int32, pin_memory=True)
    tp = torch.empty(len(rays), dtype=torch.float32, pin_memory=True)
    npn = torch.empty((len(rays), 3), dtype=torch.float32, pin_memory=True)
    m.cast_rays_and_get_normal(rp, 100.0, out=(fp, tp, npn))
    _compare(fp.numpy().view(np.uint32), tp.numpy(), npn.numpy(), fo, to, no)
    f, t, n = m.cast_rays_and_get_normal(rays, 100.0)  # pageable: staged
    _compare(f, t, n, fo, to, no)
    # device rays, pinned outputs
    fp.zero_()
    m.cast_rays_and_get_normal(rp.cuda(), 100.0, out=(fp, tp, npn))
    _compare(fp.numpy().view(np.uint32), tp.numpy(), npn.numpy(), fo, to, no)
    ctx.close()


def _grid_mesh(nx=8, nz=8, tilt=False):
    """A height field on integer grid points (heights 0..3, exact in f32), two triangles per cell
    (one diagonal), or a tilted plane: shared edges and vertices where hits tie exactly."""
    xs, zs = np.meshgrid(np.arange(nx + 1, dtype=np.float32), np.arange(nz + 1, dtype=np.float32), indexing="ij")
    h = (xs * 0.5 + zs * 0.25) if tilt else ((xs.astype(np.int64) * 7 + zs.astype(np.int64) * 3) % 4).astype(np.float32)
    v = np.stack([xs.ravel(), h.ravel().astype(np.float32), zs.ravel()], axis=1).astype(np.float32)
    idx = []
    for i in range(nx):
        for j in range(nz):
            a, b, c, d = i * (nz + 1) + j, (i + 1) * (nz + 1) + j, (i + 1) * (nz + 1) + j + 1, i * (nz + 1) + j + 1
            idx += [[a, d, b], [b, d, c]]
    return v, np.array(idx, np.uint32)


@pytest.mark.parametrize("tilt", [False, True])
def test_degenerate_rays_vs_oracle(gpu_ctx, oracle_lib, tilt):
    """Rays the reference's arithmetic treats specially, against the f32 oracle: straight down onto
    grid vertices and edges (exact toi ties between triangles: the lowest index wins), axis-aligned
    and two-zero-component directions (the slab test's zero-direction branch), horizontal rays along
    the grid lines (parallel to faces), origins on the surface (toi 0), hits at exactly max_toi
    (rejected) and the zero direction."""
    v, i = _grid_mesh(tilt=tilt)
    rays = []
    for x in np.arange(0.0, 8.01, 0.5):
        for z in np.arange(0.0, 8.01, 0.5):
            rays.append([x, 10.0, z, 0.0, -1.0, 0.0])           # vertical: vertices, edges, cell centres
            rays.append([x, 10.0, z, 0.0, -1.0, 1e-30])          # nearly vertical, denormal-free tiny component
    for y in np.arange(0.0, 3.01, 0.5):
        for k in np.arange(0.0, 8.01, 1.0):
            rays.append([-1.0, y, k, 1.0, 0.0, 0.0])             # along grid lines, one axis only
            rays.append([k, y, -1.0, 0.0, 0.0, 1.0])
            rays.append([-1.0, y, -1.0, 1.0, 0.0, 1.0])          # diagonal, zero y component
    for x in np.arange(0.25, 8.0, 1.0):
        rays.append([x, float(v[int(x) * 9, 1]) if not tilt else x * 0.5, 0.0, 0.0, -1.0, 0.0])  # on or at the surface
    rays.append([4.0, 10.0, 4.0, 0.0, 0.0, 0.0])                 # zero direction
    rays = np.array(rays, np.float32)
    m = pg.TriMesh(gpu_ctx, v, i)
    O = oracle_lib.TriMesh(v, i)
    for max_toi in (100.0, 7.0, 10.0 - 1.0):
        f, t, n = m.cast_rays_and_get_normal(rays, max_toi)
        fo, to, no = O.cast_rays_and_get_normal(rays, max_toi)
        _compare(f, t, n, fo, to, no)
        np.testing.assert_array_equal(t[fo != pg.NO_HIT].view(np.uint32), to[fo != pg.NO_HIT].view(np.uint32))
    assert int((fo != pg.NO_HIT).sum()) > len(rays) // 3
