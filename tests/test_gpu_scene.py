"""The per-frame pipeline (parrygpu_scene) against the oracle's frame loop: poses, pair sets,
per-pair manifold records and ray hits, bit-exact, with and without the CUDA graph."""
import numpy as np
import pytest

from parry_gb300 import manifold as M
from tests._contact_cases import hull_scene

pytestmark = pytest.mark.gpu


def _inputs(n, seed, n_rays=3000, extent=6.0):
    s, _ = hull_scene(n, seed, extent=extent)
    rng = np.random.default_rng(seed + 1000)
    vel = np.concatenate([rng.uniform(-5, 5, (n, 3)), rng.uniform(-1, 1, (n, 3))], axis=1).astype(np.float32)
    rays = np.concatenate([rng.uniform(-extent - 2, extent + 2, (n_rays, 3)), rng.normal(size=(n_rays, 3))], axis=1)
    rays[:, 3:] /= np.linalg.norm(rays[:, 3:], axis=1, keepdims=True)
    return s, vel, rays.astype(np.float32)


def _sorted_state(st):
    pairs = st["pairs"]
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order], M.as_words(st["manifolds"])[order] if st["manifolds"].dtype == M.MANIFOLD_DTYPE else st["manifolds"][order]


def _assert_records(gw, ww):
    np.testing.assert_array_equal(gw[:, :8], ww[:, :8])
    n = ww[:, 0].astype(np.int64)
    valid = np.arange(M.MAX_POINTS)[None, :] < n[:, None]
    gp = gw[:, 8:].reshape(len(gw), M.MAX_POINTS, 10)
    wp = ww[:, 8:].reshape(len(ww), M.MAX_POINTS, 10)
    assert np.array_equal(gp[valid], wp[valid])


@pytest.mark.parametrize("use_graph,frames", [(True, 4), (False, 3), (True, 5)])
def test_scene_matches_oracle(gpu_ctx, oracle_lib, use_graph, frames):
    import parry_gb300 as pg
    O = oracle_lib
    s, vel, rays = _inputs(600, 31)
    pred, dt = 0.1, 1.0 / 60.0
    sc = pg.Scene(gpu_ctx, s, vel, pred, 1 << 16)
    sc.set_rays(rays, 100.0)
    sc.step(dt, frames, use_graph=use_graph)
    frame, npairs = sc.info()
    assert frame == frames
    got = sc.read()
    sc.close()
    want = O.scene_frames(s, vel, pred, dt, frames, rays=rays, max_toi=100.0)
    np.testing.assert_array_equal(got["poses"], want["poses"])
    gp, gw = _sorted_state(got)
    assert npairs == len(want["pairs"]) and len(want["pairs"]) > 500
    np.testing.assert_array_equal(gp, want["pairs"])
    _assert_records(gw, want["manifolds"])
    assert int((want["manifolds"][:, 0] > 0).sum()) > 100
    np.testing.assert_array_equal(got["ray_part"], want["ray_part"])
    np.testing.assert_array_equal(got["ray_toi"], want["ray_toi"])
    np.testing.assert_array_equal(got["ray_normal"], want["ray_normal"])
    assert int((got["ray_part"] != pg.NO_HIT).sum()) > 200


def test_scene_graph_equals_eager(gpu_ctx):
    import parry_gb300 as pg
    s, vel, rays = _inputs(1200, 7, n_rays=4000, extent=8.0)
    out = []
    for g in (False, True):
        sc = pg.Scene(gpu_ctx, s, vel, 0.05, 1 << 16)
        sc.set_rays(rays, 50.0)
        sc.step(1.0 / 60.0, 6, use_graph=g)
        out.append(sc.read())
        sc.close()
    a, b = out
    np.testing.assert_array_equal(a["poses"], b["poses"])
    pa, wa = _sorted_state(a)
    pb, wb = _sorted_state(b)
    np.testing.assert_array_equal(pa, pb)
    _assert_records(wa, wb)
    np.testing.assert_array_equal(a["ray_part"], b["ray_part"])
    np.testing.assert_array_equal(a["ray_toi"], b["ray_toi"])


def test_scene_pair_capacity_is_reported(gpu_ctx):
    import parry_gb300 as pg
    s, vel, _ = _inputs(600, 3)
    sc = pg.Scene(gpu_ctx, s, vel, 0.1, 64)
    sc.step(1.0 / 60.0, 1, use_graph=False)
    with pytest.raises(pg.ParryGpuError):
        sc.info()
    sc.close()


def test_scene_mixed_eager_and_graph_frames(gpu_ctx):
    """An odd number of eager frames between graph replays flips the double buffers; the graph is
    re-captured for the new parity and the state matches an all-eager run."""
    import parry_gb300 as pg
    s, vel, rays = _inputs(500, 17, n_rays=1000)
    runs = []
    for plan in ([(1, False), (2, True), (1, False), (2, True)], [(6, False)]):
        sc = pg.Scene(gpu_ctx, s, vel, 0.1, 1 << 15)
        sc.set_rays(rays, 100.0)
        for frames, g in plan:
            sc.step(1.0 / 60.0, frames, use_graph=g)
        runs.append(sc.read())
        sc.close()
    a, b = runs
    np.testing.assert_array_equal(a["poses"], b["poses"])
    pa, wa = _sorted_state(a)
    pb, wb = _sorted_state(b)
    np.testing.assert_array_equal(pa, pb)
    _assert_records(wa, wb)
    np.testing.assert_array_equal(a["ray_part"], b["ray_part"])


@pytest.mark.parametrize("use_graph,frames", [(False, 3), (True, 4)])
def test_scene_learned_seeding_matches_oracle(gpu_ctx, oracle_lib, use_graph, frames):
    """With a network set, the scene's polyhedral pairs without a cached normal start GJK from the
    network's direction. The oracle's frame loop given the same directions (the network run on the
    frame's pair features, as the scene runs it) reproduces every pose, pair and record bit for bit;
    the seeded pairs are counted and change the GJK runs."""
    import parry_gb300 as pg
    O = oracle_lib
    s, vel, rays = _inputs(600, 41)
    pred, dt = 0.1, 1.0 / 60.0
    mlp = pg.WarmStartMLP(gpu_ctx, seed=11)

    def dirs_fn(shapes, pairs):
        return mlp.predict(mlp.features(shapes, pairs))

    sc = pg.Scene(gpu_ctx, s, vel, pred, 1 << 16)
    sc.set_rays(rays, 100.0)
    sc.set_mlp(mlp)
    sc.step(dt, frames, use_graph=use_graph)
    got = sc.read()
    seeded = sc.stats()
    sc.set_mlp(None)
    sc.close()
    want = O.scene_frames(s, vel, pred, dt, frames, rays=rays, max_toi=100.0, dirs_fn=dirs_fn)
    np.testing.assert_array_equal(got["poses"], want["poses"])
    gp, gw = _sorted_state(got)
    assert len(want["pairs"]) > 500
    np.testing.assert_array_equal(gp, want["pairs"])
    _assert_records(gw, want["manifolds"])
    np.testing.assert_array_equal(got["ray_part"], want["ray_part"])
    assert seeded["seeded_pairs"] > 0
    # the first frame seeds every polyhedral pair; the plain first frame differs in GJK iterations
    runs = []
    for with_mlp in (True, False):
        sc = pg.Scene(gpu_ctx, s, vel, pred, 1 << 16)
        if with_mlp:
            sc.set_mlp(mlp)
        sc.step(dt, 1, use_graph=False)
        runs.append(sc.stats())
        sc.close()
    from parry_gb300.shapes import BALL, CUBOID, CAPSULE
    t = s.arrays()[0]
    pf = O.scene_frames(s, vel, pred, dt, 1)["pairs"]
    ta, tb = t[pf[:, 0]], t[pf[:, 1]]
    poly = (ta != BALL) & (tb != BALL) & ~((ta == tb) & ((ta == CUBOID) | (ta == CAPSULE)))
    assert runs[0]["seeded_pairs"] == int(poly.sum()) > 0 and runs[1]["seeded_pairs"] == 0
    assert runs[0]["gjk_iters"] != runs[1]["gjk_iters"]


def _grid_rays(n, extent, seed):
    """Random rays plus axis-aligned ones (zero direction components), rays from outside the shapes'
    bounds, and a zero-direction ray."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-extent - 5, extent + 5, (n, 3))
    d = rng.normal(size=(n, 3))
    d[: n // 8] = np.eye(3)[rng.integers(0, 3, n // 8)] * rng.choice([-1.0, 1.0], (n // 8, 1))
    d[n // 8: n // 4, rng.integers(0, 3)] = 0.0
    d[-1] = 0.0
    o[n // 4: n // 4 + n // 16] *= 4.0
    nz = np.linalg.norm(d, axis=1, keepdims=True)
    d = np.where(nz > 0, d / np.maximum(nz, 1e-30), d)
    return np.concatenate([o, d], axis=1).astype(np.float32)


@pytest.mark.parametrize("giant", [False, True])
def test_scene_ray_grid_matches_bvh_and_oracle(oracle_lib, giant):
    """The frame pipeline's rays through the per-frame uniform grid and through the BVH give the same
    answers, equal to the oracle's, for random, axis-aligned, outside-origin and zero-direction rays.
    With every cuboid 3 times larger the entries outgrow the grid's capacity, the grid reports
    itself unusable and the BVH kernel casts the rays: same answers again."""
    import parry_gb300 as pg
    O = oracle_lib
    s, vel, _ = _inputs(900, 53, extent=7.0)
    if giant:
        t, prm, pos, pool = s.arrays()
        poly = s.polyhedra()
        from parry_gb300.shapes import CUBOID
        t = t.copy()
        prm = prm.copy()
        prm[t == CUBOID, :3] *= 3.0
        s = pg.ShapeSet.from_arrays(t, prm, pos, pool, poly)
    rays = _grid_rays(6000, 7.0, 5)
    out = []
    for mode in (1, 2):
        ctx = pg.Context(0, scene_ray_grid=mode)
        sc = pg.Scene(ctx, s, vel, 0.1, 1 << 20)
        sc.set_rays(rays, 40.0)
        sc.step(1.0 / 60.0, 3, use_graph=True)
        out.append(sc.read())
        sc.close()
        ctx.close()
    a, b = out
    for key in ("ray_part", "ray_toi", "ray_normal"):
        np.testing.assert_array_equal(a[key], b[key])
    want = O.scene_frames(s, vel, 0.1, 1.0 / 60.0, 3, rays=rays, max_toi=40.0)
    np.testing.assert_array_equal(a["ray_part"], want["ray_part"])
    np.testing.assert_array_equal(a["ray_toi"], want["ray_toi"])
    np.testing.assert_array_equal(a["ray_normal"], want["ray_normal"])
    assert int((a["ray_part"] != pg.NO_HIT).sum()) > 300


def test_scene_ray_grid_candidate_overflow(oracle_lib):
    """A row of 800 balls, cuboids, capsules and hulls along every ray: the grid walk's candidate
    lists (4 per ray + 1024 entries) overflow in its staged batches, and the affected rays are recast
    by the single-kernel path. Same answers as the BVH path and the oracle."""
    import parry_gb300 as pg
    O = oracle_lib
    s = pg.ShapeSet()
    rng = np.random.default_rng(9)
    pts = rng.normal(size=(24, 3))
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    for i in range(800):
        pose = (0.0, 0.0, 0.0, 1.0, 2.0 * i, 0.0, 0.0)
        kind = i % 4
        if kind == 0:
            s.add_ball(0.45, pose)
        elif kind == 1:
            s.add_cuboid((0.3, 0.4, 0.35), pose)
        elif kind == 2:
            s.add_capsule(0.4, 0.3, pose)
        else:
            s.add_convex(pts * 0.5, pose)
    n = 64
    o = np.stack([np.full(n, -5.0), rng.uniform(-0.2, 0.2, n), rng.uniform(-0.2, 0.2, n)], 1)
    d = np.tile([1.0, 0.0, 0.0], (n, 1)) + rng.normal(scale=1e-3, size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    vel = np.zeros((800, 6), np.float32)
    out = []
    for mode in (1, 2):
        ctx = pg.Context(0, scene_ray_grid=mode)
        sc = pg.Scene(ctx, s, vel, 0.1, 1 << 16)
        sc.set_rays(rays, 2000.0)
        sc.step(1.0 / 60.0, 2, use_graph=False)
        out.append(sc.read())
        sc.close()
        ctx.close()
    a, b = out
    want = O.scene_frames(s, vel, 0.1, 1.0 / 60.0, 2, rays=rays, max_toi=2000.0)
    for key in ("ray_part", "ray_toi", "ray_normal"):
        np.testing.assert_array_equal(a[key], b[key])
        np.testing.assert_array_equal(a[key], want[key])
    assert np.all(a["ray_part"] != pg.NO_HIT)


def test_scene_read_into_pinned_buffers(gpu_ctx):
    """Scene.read into caller-provided (pinned) buffers gives the same state as a fresh read."""
    import torch
    import parry_gb300 as pg
    s, vel, rays = _inputs(700, 61, n_rays=2000)
    sc = pg.Scene(gpu_ctx, s, vel, 0.1, 1 << 15)
    sc.set_rays(rays, 100.0)
    sc.step(1.0 / 60.0, 2, use_graph=True)
    a = sc.read()
    pin = {"poses": torch.empty((700, 7), dtype=torch.float32, pin_memory=True),
           "pairs": torch.empty((1 << 15, 2), dtype=torch.int32, pin_memory=True),
           "manifolds": torch.empty((1 << 15, M.RECORD_WORDS), dtype=torch.int32, pin_memory=True),
           "ray_part": torch.empty(2000, dtype=torch.int32, pin_memory=True),
           "ray_toi": torch.empty(2000, dtype=torch.float32, pin_memory=True),
           "ray_normal": torch.empty((2000, 3), dtype=torch.float32, pin_memory=True)}
    b = sc.read(out=pin)
    sc.close()
    np.testing.assert_array_equal(a["poses"], b["poses"].numpy())
    np.testing.assert_array_equal(a["pairs"], b["pairs"].numpy().view(np.uint32))
    np.testing.assert_array_equal(M.as_words(a["manifolds"]), b["manifolds"].numpy().view(np.uint32))
    np.testing.assert_array_equal(a["ray_part"], b["ray_part"].numpy().view(np.uint32))
    np.testing.assert_array_equal(a["ray_toi"], b["ray_toi"].numpy())
    np.testing.assert_array_equal(a["ray_normal"], b["ray_normal"].numpy())


def _pinned(n, cap, n_rays):
    import torch
    return {"poses": torch.empty((n, 7), dtype=torch.float32, pin_memory=True),
            "pairs": torch.empty((cap, 2), dtype=torch.int32, pin_memory=True),
            "manifolds": torch.empty((cap, M.RECORD_WORDS), dtype=torch.int32, pin_memory=True),
            "ray_part": torch.empty(n_rays, dtype=torch.int32, pin_memory=True),
            "ray_toi": torch.empty(n_rays, dtype=torch.float32, pin_memory=True),
            "ray_normal": torch.empty((n_rays, 3), dtype=torch.float32, pin_memory=True)}


def _assert_same_read(a, b):
    """A read of one scene (numpy) against a read of its twin into pinned buffers: pairs come in
    append order, so they are compared as sets, each with its record."""
    np.testing.assert_array_equal(a["poses"], b["poses"].numpy())
    pa, ra = _sorted_state(a)
    pb, rb = _sorted_state({"pairs": b["pairs"].numpy().view(np.uint32), "manifolds": b["manifolds"].numpy().view(np.uint32)})
    np.testing.assert_array_equal(pa, pb)
    _assert_records(rb, ra)
    np.testing.assert_array_equal(a["ray_part"], b["ray_part"].numpy().view(np.uint32))
    np.testing.assert_array_equal(a["ray_toi"], b["ray_toi"].numpy())
    np.testing.assert_array_equal(a["ray_normal"], b["ray_normal"].numpy())


def test_scene_async_read_overlaps_next_frames(gpu_ctx):
    """Scene.read(wait=False) copies a frame's outputs while the next frames run: after read_wait the
    buffers hold that frame's outputs (a twin scene read synchronously gives the same), the frames
    after it are unchanged by the read, and graph replays after a read stay correct."""
    import parry_gb300 as pg
    s, vel, rays = _inputs(700, 71, n_rays=2000)
    dt, cap = 1.0 / 60.0, 1 << 15
    a = pg.Scene(gpu_ctx, s, vel, 0.1, cap)
    b = pg.Scene(gpu_ctx, s, vel, 0.1, cap)
    for sc in (a, b):
        sc.set_rays(rays, 100.0)
    pin = _pinned(700, cap, 2000)
    for frame in range(4):
        a.step(dt, 1, use_graph=False)
        b.step(dt, 1, use_graph=False)
        want = b.read()
        got = a.read(out=pin, wait=False)
        a.step(dt, 1, use_graph=False)  # runs while the copies proceed
        a.read_wait()
        _assert_same_read(want, got)
        b.step(dt, 1, use_graph=False)
        _assert_same_read(b.read(), a.read(out=_pinned(700, cap, 2000)))
    # a read followed by graph replays, then an eager frame
    got = a.read(out=pin, wait=False)
    want = b.read()
    a.step(dt, 4, use_graph=True)
    b.step(dt, 4, use_graph=True)
    a.read_wait()
    _assert_same_read(want, got)
    a.step(dt, 1, use_graph=False)
    b.step(dt, 1, use_graph=False)
    _assert_same_read(b.read(), a.read(out=_pinned(700, cap, 2000)))
    assert len(want["pairs"]) > 100 and int((want["ray_part"] != pg.NO_HIT).sum()) > 100
    a.close()
    b.close()
