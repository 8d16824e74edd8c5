"""Parity of the CUDA LBVH (build, refit, self pairs, tree-vs-tree pairs) with the oracle:
pair sets must be identical as sorted sets; the tree must pass the reference's well-formedness
checks (restated in tests/_helpers.py)."""
import numpy as np
import pytest

import parry_gb300 as pg
from tests._helpers import assert_well_formed, brute_force_pairs, random_aabbs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 64, 1000, 20000])
def test_build_well_formed_and_self_pairs(gpu_ctx, oracle_lib, n):
    a = random_aabbs(n, seed=n + 1, extent=30.0) if n else np.zeros((0, 6), np.float32)
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    assert b.leaf_count() == n
    assert_well_formed(b.nodes(), n)
    got = b.traverse_bvtt_single_tree()
    if n >= 2:
        want = oracle_lib.canonical_sorted_pairs(oracle_lib.Bvh(a).traverse_bvtt_single_tree())
        np.testing.assert_array_equal(got, want)
        if n <= 5000:
            np.testing.assert_array_equal(got, brute_force_pairs(a))
    else:
        assert len(got) == 0


def test_duplicate_centroids(gpu_ctx, oracle_lib):
    """Identical Morton codes (all boxes at the same centre) still give a valid tree and all pairs."""
    a = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (300, 1))
    a[::2, 3:] += 0.5
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    assert_well_formed(b.nodes(), 300)
    got = b.traverse_bvtt_single_tree()
    assert len(got) == 300 * 299 // 2
    np.testing.assert_array_equal(got, brute_force_pairs(a))


def test_refit(gpu_ctx, oracle_lib):
    a = random_aabbs(5000, seed=77, extent=40.0)
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    rng = np.random.default_rng(5)
    d = rng.uniform(-2, 2, size=(5000, 3)).astype(np.float32)
    a2 = a + np.concatenate([d, d], 1)
    b.refit(a2)
    assert_well_formed(b.nodes(), 5000)
    np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), brute_force_pairs(a2))


@pytest.mark.parametrize("na,nb", [(1, 1), (1, 2), (2, 1), (2, 2), (3, 5), (700, 900)])
def test_leaf_pairs(gpu_ctx, oracle_lib, na, nb):
    a = random_aabbs(na, seed=na * 7 + 1, extent=10.0)
    b = random_aabbs(nb, seed=nb * 13 + 2, extent=10.0)
    ga, gb = pg.Bvh.from_leaves(gpu_ctx, a), pg.Bvh.from_leaves(gpu_ctx, b)
    got = ga.leaf_pairs(gb)
    want = oracle_lib.sorted_pairs(oracle_lib.Bvh(a).leaf_pairs(oracle_lib.Bvh(b)))
    if na > 2 or nb > 2:
        # root-level quirk pairs depend on each tree's root children: compare the checked part
        mn_a, mx_a, mn_b, mx_b = a[:, None, :3], a[:, None, 3:], b[None, :, :3], b[None, :, 3:]
        ok = np.all(mn_a <= mx_b, -1) & np.all(mx_a >= mn_b, -1)
        strip = lambda p: p[ok[p[:, 0], p[:, 1]]] if len(p) else p
        np.testing.assert_array_equal(strip(got), strip(want))
    else:
        np.testing.assert_array_equal(got, want)


def test_capacity_exceeded_reports_count(gpu_ctx):
    import ctypes as C
    a = random_aabbs(2000, seed=3, extent=5.0)
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    full = b.traverse_bvtt_single_tree()
    assert len(full) > 10
    out = np.zeros((10, 2), np.uint32)
    n = C.c_uint64(0)
    st = pg.lib().parrygpu_bvh_self_pairs(gpu_ctx.handle, b._h, C.c_void_p(out.ctypes.data), 10, C.byref(n), 1)
    assert st == 3 and n.value == len(full)
