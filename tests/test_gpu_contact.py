"""Parity of the CUDA query::contact path (through the C ABI) with the oracle's f32 restatement:
has-contact decisions identical; points, normals and depth within 1e-5 (relative, with an absolute
floor of 1e-5 for values near zero); error against the f64 oracle stated."""
import numpy as np
import pytest

import parry_gb300 as pg
from parry_gb300 import workloads as W
from tests import _contact_cases as CC

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _compare(has, out, ho, oo, what=""):
    np.testing.assert_array_equal(has, ho, err_msg=f"has_contact differs {what}")
    m = ho == 1
    np.testing.assert_allclose(out[m], oo[m], rtol=TOL, atol=TOL, err_msg=what)


def test_known_answers(gpu_ctx, oracle_lib):
    s, pairs, c = CC.cuboid_epa()
    has, out = pg.contacts(gpu_ctx, s, pairs, c["prediction"])
    assert has.all()
    for k, case in enumerate(c["cases"]):
        assert out[k, 12] == np.float32(case["expect_dist"])
        np.testing.assert_array_equal(out[k, 6:9], np.array(case["expect_normal1"], np.float32))
    s, pairs, c = CC.triangle_touch()
    has, out = pg.contacts(gpu_ctx, s, pairs, c["prediction"])
    assert has[0] == 1 and abs(out[0, 1] - c["expect_point1_y"]) <= c["tolerance"]
    assert abs(out[0, 0] - c["expect_point1_x"]) <= c["tolerance"]
    s, pairs, c = CC.ball_ball()
    for case in c["cases"]:
        has, out = pg.contacts(gpu_ctx, s, pairs, case["prediction"])
        assert (has[0] == 0) if case["expect"] is None else (has[0] == 1 and 0 < out[0, 12] <= case["prediction"])
    s, pairs, c = CC.ball_cuboid()
    has, out = pg.contacts(gpu_ctx, s, pairs, c["prediction"])
    assert has[0] == 1 and out[0, 12] <= 0 and has[1] == 1 and out[1, 12] >= 0 and has[2] == 0


def test_hull_pairs_vs_oracle(gpu_ctx, oracle_lib):
    s, pairs = W.hull_pairs(50_000, seed=11)
    has, out, st = pg.contacts(gpu_ctx, s, pairs, 0.0, want_stats=True)
    ho, oo, sto = oracle_lib.contacts(s, pairs, 0.0)
    _compare(has, out, ho, oo, "hull pairs")
    assert st["gjk_iters"] == sto["gjk_iters"] and st["epa_iters"] == sto["epa_iters"]
    h64, o64, _ = oracle_lib.contacts(s, pairs, 0.0, precision="f64")
    m = (ho == 1) & (h64 == 1)
    err = np.abs(out[m, 12].astype(np.float64) - o64[m, 12])
    print(f"\ndepth abs err vs f64 oracle: max {err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")


def test_mixed_shapes_vs_oracle(gpu_ctx, oracle_lib):
    """Balls, cuboids, capsules, hulls and triangles in every combination, with prediction."""
    rng = np.random.default_rng(7)
    s = pg.ShapeSet()
    pool, first, count = W.ellipsoid_hulls(64, seed=5, stream=1, nmin=8, nmax=64)
    n = 400
    for i in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pose = pg.shapes.pose7(rng.uniform(-3, 3, 3), q)
        t = i % 5
        if t == 0:
            s.add_ball(rng.uniform(0.3, 2.0), pose)
        elif t == 1:
            s.add_cuboid(rng.uniform(0.3, 2.0, 3), pose)
        elif t == 2:
            s.add_capsule(rng.uniform(0.2, 1.5), rng.uniform(0.2, 1.0), pose)
        elif t == 3:
            h = i % 64
            s.add_convex(pool[first[h]:first[h] + count[h]], pose)
        else:
            s.add_triangle(*rng.uniform(-1.5, 1.5, (3, 3)), pose)
    pairs = np.array([(a, b) for a in range(0, n, 3) for b in range(1, n, 7) if a != b], np.uint32)
    for pred in (0.0, 0.25):
        has, out = pg.contacts(gpu_ctx, s, pairs, pred)
        ho, oo, _ = oracle_lib.contacts(s, pairs, pred)
        _compare(has, out, ho, oo, f"mixed shapes prediction {pred}")
        assert ho.sum() > 100


def test_init_dir_warm_start(gpu_ctx, oracle_lib):
    s, pairs = W.hull_pairs(20_000, seed=12)
    rng = np.random.default_rng(1)
    d = rng.normal(size=(len(pairs), 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    has, out = pg.contacts(gpu_ctx, s, pairs, 0.0, init_dirs=d)
    ho, oo, _ = oracle_lib.contacts(s, pairs, 0.0, init_dirs=d)
    _compare(has, out, ho, oo, "init_dir")


def test_shape_aabbs(gpu_ctx, oracle_lib):
    s = W.broadphase_shapes(20_000, seed=3)
    for margin in (0.0, 0.05):
        np.testing.assert_array_equal(pg.shape_aabbs(gpu_ctx, s, margin), oracle_lib.shape_aabbs(s, margin))


def test_broadphase_pipeline(gpu_ctx, oracle_lib):
    """Shape AABBs loosened by prediction/2 -> LBVH -> all overlapping pairs -> query::contact."""
    s = W.broadphase_shapes(131072)
    a = pg.shape_aabbs(gpu_ctx, s, 0.05)
    bvh = pg.Bvh.from_leaves(gpu_ctx, a)
    pairs = bvh.traverse_bvtt_single_tree()
    want = oracle_lib.canonical_sorted_pairs(oracle_lib.Bvh(oracle_lib.shape_aabbs(s, 0.05)).traverse_bvtt_single_tree())
    np.testing.assert_array_equal(pairs, want)
    has, out = pg.contacts(gpu_ctx, s, pairs, 0.1)
    ho, oo, _ = oracle_lib.contacts(s, pairs, 0.1)
    _compare(has, out, ho, oo, "broadphase contacts")
    print(f"\n{len(pairs)} candidate pairs, {int(ho.sum())} contacts")


def test_autotune_contacts_keeps_answers(oracle_lib):
    ctx = pg.Context(0)
    s, pairs = W.hull_pairs(8192, seed=17)
    cfg = pg.autotune_contacts(ctx, s, pairs, 0.0, reps=1)
    assert cfg["epa_blocks_per_sm"] in (4, 6, 8, 12, 16) and ctx.config == cfg
    assert cfg["contact_warp_cost"] in (256, 512, 1024) and cfg["contact_epa_inline"] in (1, 2)
    has, out = pg.contacts(ctx, s, pairs, 0.0)
    ho, oo, _ = oracle_lib.contacts(s, pairs, 0.0)
    _compare(has, out, ho, oo, "after autotune")
    ctx.close()


def test_mixed_shapes_and_long_epa(gpu_ctx, oracle_lib):
    """Hulls mixed with balls, cuboids and capsules; includes a capsule-capsule pair whose EPA runs
    all 100 expansions and builds 512 faces (rounded supports never converge exactly)."""
    from parry_gb300.shapes import ShapeSet, CAPSULE
    s, pairs = W.mixed_contact_pairs(200_000, seed=23)
    has, out, st = pg.contacts(gpu_ctx, s, pairs, 0.0, want_stats=True)
    ho, oo, sto = oracle_lib.contacts(s, pairs, 0.0)
    _compare(has, out, ho, oo, "mixed shapes")
    assert st["epa_iters"] == sto["epa_iters"]
    types = np.array([CAPSULE, CAPSULE], np.uint32)
    params = np.array([[0.9470748, 0.28093398, 0, 0], [0.80303407, 0.6510845, 0, 0]], np.float32)
    poses = np.array([[0, 0, 0, 1, 0, 0, 0],
                      [-0.30348304, -0.23253627, -0.85818106, 0.3425641, -0.5920257, -0.42291966, -0.22780326]], np.float32)
    s2 = ShapeSet.from_arrays(types, params, poses)
    p2 = np.array([[0, 1]], np.uint32)
    has, out, st = pg.contacts(gpu_ctx, s2, p2, 0.0, want_stats=True)
    ho, oo, sto = oracle_lib.contacts(s2, p2, 0.0)
    assert sto["epa_max_faces"] >= 500 and st["epa_iters"] == sto["epa_iters"] == 101
    _compare(has, out, ho, oo, "capsule pair with 512 EPA faces")


@pytest.mark.parametrize("warp_cost,epa_inline", [(2, 2), (100, 2), (300, 1), (4096, 1)])
def test_warp_per_pair_path_vs_oracle(oracle_lib, warp_cost, epa_inline):
    """Pairs whose support-scan cost reaches contact_warp_cost run one warp per pair (hulls staged in
    shared memory by bulk copies, lane-parallel support scans, GJK and EPA in shared memory); the
    others one thread per pair, with EPA right after GJK in the same thread (epa_inline 1) or through
    the queue (2): the answers and iteration counts are the oracle's, with and without init_dir, with
    prediction, and on mixed shapes (ball pairs in the warp bin fall back to one lane)."""
    ctx = pg.Context(0, contact_warp_cost=warp_cost, contact_epa_inline=epa_inline)
    try:
        s, pairs = W.hull_pairs(40_000, seed=31)
        has, out, st = pg.contacts(ctx, s, pairs, 0.0, want_stats=True)
        ho, oo, sto = oracle_lib.contacts(s, pairs, 0.0)
        _compare(has, out, ho, oo, f"hull pairs, warp cost {warp_cost}")
        assert (st["gjk_iters"], st["epa_iters"], st["epa_calls"]) == (sto["gjk_iters"], sto["epa_iters"], sto["epa_calls"])
        rng = np.random.default_rng(4)
        d = rng.normal(size=(len(pairs), 3)).astype(np.float32)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        dirs = np.zeros((len(pairs), 3), np.float32)
        has, out = pg.contacts(ctx, s, pairs, 0.05, init_dirs=d, final_dirs=dirs)
        ho, oo, _ = oracle_lib.contacts(s, pairs, 0.05, init_dirs=d)
        _compare(has, out, ho, oo, "init_dir + prediction")
        dirs0 = np.zeros_like(dirs)
        ctx0 = pg.Context(0, contact_warp_cost=4096)
        pg.contacts(ctx0, s, pairs, 0.05, init_dirs=d, final_dirs=dirs0)
        ctx0.close()
        np.testing.assert_array_equal(dirs, dirs0)
        s, pairs = W.mixed_contact_pairs(60_000, seed=29)
        has, out, st = pg.contacts(ctx, s, pairs, 0.0, want_stats=True)
        ho, oo, sto = oracle_lib.contacts(s, pairs, 0.0)
        _compare(has, out, ho, oo, "mixed shapes")
        assert st["epa_iters"] == sto["epa_iters"]
    finally:
        ctx.close()


@pytest.mark.parametrize("shuffle", [False, True])
def test_pipelined_host_buffers_match_device_buffers(gpu_ctx, shuffle):
    """A large batch from host shapes runs in chunks while the vertex pool goes up in pieces (pairs
    in shape order, and shuffled so that the first chunk needs the whole pool): has_contact, the
    contacts and the final directions equal those of the same call on device buffers, bit for bit,
    from pageable and from pinned host memory."""
    import torch
    s, pairs = W.hull_pairs(300_000, seed=21)
    if shuffle:
        pairs = np.ascontiguousarray(pairs[np.random.default_rng(3).permutation(len(pairs))])
    k = len(pairs)
    dirs = np.random.default_rng(4).normal(size=(k, 3)).astype(np.float32)
    arrays = [np.ascontiguousarray(a) for a in s.arrays()]
    arrays[0] = arrays[0].view(np.int32)
    dev = tuple(torch.from_numpy(a).cuda() for a in arrays)
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    ddirs = torch.from_numpy(dirs).cuda()
    dfin = torch.empty((k, 3), dtype=torch.float32, device="cuda")
    dh, dr = pg.contacts(gpu_ctx, dev, dpairs, 0.0, init_dirs=ddirs, final_dirs=dfin)
    torch.cuda.synchronize()
    dh, dr, dfin = dh.cpu().numpy(), dr.cpu().numpy(), dfin.cpu().numpy()
    assert 0.3 < dh.mean() < 0.95
    # pageable host memory
    fin = np.empty((k, 3), np.float32)
    hh, hr = pg.contacts(gpu_ctx, s, pairs, 0.0, init_dirs=dirs, final_dirs=fin)
    np.testing.assert_array_equal(hh, dh)
    np.testing.assert_array_equal(hr.view(np.uint32), dr.view(np.uint32))
    np.testing.assert_array_equal(fin.view(np.uint32), dfin.view(np.uint32))
    # pinned host memory, outputs into caller buffers
    host = tuple(torch.from_numpy(a).pin_memory() for a in arrays)
    hp = torch.from_numpy(pairs.view(np.int32)).pin_memory()
    hd = torch.from_numpy(dirs).pin_memory()
    ph = torch.empty(k, dtype=torch.uint8, pin_memory=True)
    pr = torch.empty((k, 13), dtype=torch.float32, pin_memory=True)
    pf = torch.empty((k, 3), dtype=torch.float32, pin_memory=True)
    pg.contacts(gpu_ctx, host, hp, 0.0, init_dirs=hd, out=(ph, pr), final_dirs=pf)
    np.testing.assert_array_equal(ph.numpy(), dh)
    np.testing.assert_array_equal(pr.numpy().view(np.uint32), dr.view(np.uint32))
    np.testing.assert_array_equal(pf.numpy().view(np.uint32), dfin.view(np.uint32))


def test_degenerate_contacts_vs_oracle(gpu_ctx, oracle_lib):
    """Configurations the reference's branches single out, against the f32 oracle: coincident
    shapes (same pose), cuboids face to face at distance exactly 0 and at exactly the prediction,
    a ball centred inside a cuboid and at a cuboid's corner, balls touching, capsules whose axes
    cross, a flat (coplanar) hull and one with repeated points, coplanar triangles, and every pair
    the other way round (ball first / ball second paths)."""
    I = pg.shapes.pose7([0, 0, 0], [0, 0, 0, 1])

    def at(x, y=0.0, z=0.0, q=(0, 0, 0, 1)):
        return pg.shapes.pose7([x, y, z], q)
    s = pg.ShapeSet()
    s.add_cuboid([1, 1, 1], I)                                   # 0
    s.add_cuboid([1, 1, 1], I)                                   # 1 coincident with 0
    s.add_cuboid([1, 1, 1], at(2.0))                             # 2 face to face with 0, distance 0
    s.add_cuboid([1, 1, 1], at(2.25))                            # 3 distance 0.25 from 0
    s.add_ball(0.5, I)                                           # 4 centred inside 0
    s.add_ball(0.5, at(1.0, 1.0, 1.0))                           # 5 centred on a corner of 0
    s.add_ball(1.0, at(3.0))                                     # 6
    s.add_ball(1.0, at(5.0))                                     # 7 touching 6
    s.add_capsule(1.0, 0.5, I)                                   # 8 along y
    s.add_capsule(1.0, 0.5, at(0.0, 0.0, 0.0, (0.0, 0.0, np.sqrt(0.5), np.sqrt(0.5))))  # 9 along x, axes cross
    sq = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1], [0, 0, 0]], np.float32)
    s.add_convex(sq, at(0.0, 1.0))                               # 10 flat hull on top of 0
    rep = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 0], [0, 1, 0]], np.float32)
    s.add_convex(rep, at(0.5, 0.5, 0.5))                         # 11 repeated points, inside 0
    s.add_triangle([-1, 0, -1], [1, 0, -1], [0, 0, 1], I)        # 12
    s.add_triangle([-1, 0, -1], [1, 0, -1], [0, 0, 1], I)        # 13 coplanar with 12
    s.add_triangle([-1, 0, 1], [1, 0, 1], [0, 0, -1], at(0.0, 1.0))  # 14 on the top face of 0
    n = 15
    pairs = np.array([(a, b) for a in range(n) for b in range(n) if a != b], np.uint32)
    for pred in (0.0, 0.25, 1.0):
        has, out = pg.contacts(gpu_ctx, s, pairs, pred)
        ho, oo, _ = oracle_lib.contacts(s, pairs, pred)
        _compare(has, out, ho, oo, f"degenerate configurations, prediction {pred}")
    assert ho.sum() > len(pairs) // 3
