"""The reference's serialised Bvh (nodes, parents, leaf_node_indices) and leaf edits on the GPU:
export matches the links recomputed from the nodes; a tree built by the oracle's restatement of
parry's binned builder imports and answers pair queries like brute force; insert / update / remove
leave a tree whose pairs and refits match brute force over the edited leaf set."""
import numpy as np
import pytest

import parry_gb300 as pg
from tests._helpers import assert_well_formed, brute_force_pairs, random_aabbs, serialized_links

pytestmark = pytest.mark.gpu

NONE = np.uint64(2**64 - 1)


def _pairs_by_id(ids: np.ndarray, aabbs: np.ndarray) -> np.ndarray:
    """Brute-force pairs over rows, reported as (min id, max id), sorted."""
    p = brute_force_pairs(aabbs)
    a, b = ids[p[:, 0]], ids[p[:, 1]]
    out = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1).astype(np.uint32)
    return out[np.lexsort((out[:, 1], out[:, 0]))] if len(out) else out.reshape(0, 2)


@pytest.mark.parametrize("n", [1, 2, 3, 1000])
def test_export_matches_links(gpu_ctx, n):
    a = random_aabbs(n, seed=11 + n, extent=20.0)
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    nodes, parents, leaves = b.serialize(leaf_capacity=n + 5)
    np.testing.assert_array_equal(nodes.view(np.uint32), b.nodes().view(np.uint32))
    want_parents, want_leaves = serialized_links(nodes)
    np.testing.assert_array_equal(parents, want_parents)
    assert sorted(want_leaves) == list(range(n))
    for i in range(n):
        assert leaves[i] == want_leaves[i]
    assert np.all(leaves[n:] == NONE)
    b.close()


@pytest.mark.parametrize("n", [1, 2, 7, 3000])
def test_import_parry_binned_tree(gpu_ctx, oracle_lib, n):
    """A tree from parry's binned build (restated by the oracle) loads as is and gives the same
    pairs as brute force; exporting it returns the same nodes and the reference's links."""
    a = random_aabbs(n, seed=70 + n, extent=25.0)
    ref = oracle_lib.Bvh(a)
    nodes = np.ascontiguousarray(ref.nodes()).view(np.float32).reshape(-1, 16)
    b = pg.Bvh.from_serialized(gpu_ctx, nodes)
    assert b.leaf_count() == n
    if n >= 2:
        np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), brute_force_pairs(a))
    out_nodes, parents, leaves = b.serialize()
    np.testing.assert_array_equal(out_nodes.view(np.uint32), nodes.view(np.uint32))
    want_parents, want_leaves = serialized_links(nodes)
    np.testing.assert_array_equal(parents, want_parents)
    assert all(leaves[i] == want_leaves[i] for i in range(n))
    # refit keeps working on the imported topology
    a2 = a + np.float32(0.5)
    b.refit(a2)
    if n >= 2:
        np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), brute_force_pairs(a2))
    assert_well_formed(b.nodes(), n)
    b.close()


def test_import_rejects_malformed(gpu_ctx, oracle_lib):
    a = random_aabbs(50, seed=5, extent=10.0)
    nodes = np.ascontiguousarray(oracle_lib.Bvh(a).nodes()).view(np.float32).reshape(-1, 16).copy()
    u = nodes.view(np.uint32)
    bad = nodes.copy()
    bv = bad.view(np.uint32)
    internal = np.nonzero((u[:, 7] & 0x3FFFFFFF) > 1)[0]
    bv[internal[0], 3] = len(nodes) + 3  # child index out of range
    with pytest.raises(pg.ParryGpuError):
        pg.Bvh.from_serialized(gpu_ctx, bad)
    bad = nodes.copy()
    bv = bad.view(np.uint32)
    bv[0, 7] = (bv[0, 7] & 0xC0000000) | ((u[0, 7] & 0x3FFFFFFF) + 1)  # leaf counts do not add up
    with pytest.raises(pg.ParryGpuError):
        pg.Bvh.from_serialized(gpu_ctx, bad)
    bad = nodes.copy()
    bv = bad.view(np.uint32)
    leaf = np.nonzero((u[:, 7] & 0x3FFFFFFF) == 1)[0]
    bv[leaf[0], 3] = 0xFFFFFFFF  # leaf index above PARRYGPU_MAX_LEAF_INDEX (its row count would wrap to 0)
    with pytest.raises(pg.ParryGpuError):
        pg.Bvh.from_serialized(gpu_ctx, bad)
    ok = pg.Bvh.from_serialized(gpu_ctx, nodes)  # the context is still usable
    assert ok.leaf_count() == 50
    # an insert with an out-of-range leaf index is refused and leaves the tree as it was
    with pytest.raises(pg.ParryGpuError):
        ok.insert(a[:2], np.array([3, 0xFFFFFFFF], np.uint32))
    assert ok.leaf_count() == 50 and ok.id_bound() == 50
    np.testing.assert_array_equal(ok.traverse_bvtt_single_tree(), brute_force_pairs(a))
    ok.close()


def test_insert_update_remove(gpu_ctx):
    rng = np.random.default_rng(3)
    n = 2000
    a = random_aabbs(n, seed=8, extent=30.0)
    table = {i: a[i] for i in range(n)}
    b = pg.Bvh.from_leaves(gpu_ctx, a)
    # insert new indices with gaps, and update some existing ones (the last row of an index wins)
    new_ids = np.concatenate([np.arange(5000, 5600, 3), rng.choice(n, 100, replace=False), [7, 7]]).astype(np.uint32)
    new_boxes = random_aabbs(len(new_ids), seed=9, extent=30.0)
    b.insert(new_boxes, new_ids)
    for i, box in zip(new_ids, new_boxes):
        table[int(i)] = box
    ids = np.array(sorted(table), np.uint32)
    boxes = np.stack([table[int(i)] for i in ids])
    assert b.leaf_count() == len(ids)
    assert_well_formed(b.nodes(), len(ids), leaf_data_is_index=False)
    np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), _pairs_by_id(ids, boxes))
    # remove some indices (and some that name no leaf)
    gone = np.concatenate([rng.choice(ids, 300, replace=False), [4999, 123456]]).astype(np.uint32)
    b.remove(gone)
    for i in gone:
        table.pop(int(i), None)
    ids = np.array(sorted(table), np.uint32)
    boxes = np.stack([table[int(i)] for i in ids])
    assert b.leaf_count() == len(ids)
    np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), _pairs_by_id(ids, boxes))
    # refit with AABBs indexed by leaf index
    bound = int(ids.max()) + 1
    assert b.id_bound() == bound
    full = np.zeros((bound, 6), np.float32)
    moved = boxes + rng.uniform(-1, 1, size=(len(ids), 1)).astype(np.float32)
    full[ids] = moved
    b.refit(full)
    np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), _pairs_by_id(ids, moved))
    _, _, leaves = b.serialize()
    assert np.all((leaves != NONE) == np.isin(np.arange(bound), ids))
    # removing everything leaves an empty tree; inserting again starts over
    b.remove(ids)
    assert b.leaf_count() == 0
    b.insert(a[:3], np.array([10, 20, 30], np.uint32))
    assert b.leaf_count() == 3
    b.close()


def test_edit_imported_tree(gpu_ctx, oracle_lib):
    """A tree imported from parry's binned layout takes inserts and removals like a built one."""
    a = random_aabbs(500, seed=21, extent=15.0)
    nodes = np.ascontiguousarray(oracle_lib.Bvh(a).nodes()).view(np.float32).reshape(-1, 16)
    b = pg.Bvh.from_serialized(gpu_ctx, nodes)
    extra = random_aabbs(50, seed=22, extent=15.0)
    b.insert(extra, np.arange(1000, 1050, dtype=np.uint32))
    b.remove(np.arange(0, 500, 5, dtype=np.uint32))
    ids = np.array(sorted(set(range(500)) - set(range(0, 500, 5))) + list(range(1000, 1050)), np.uint32)
    boxes = np.concatenate([a[ids[ids < 500]], extra])
    np.testing.assert_array_equal(b.traverse_bvtt_single_tree(), _pairs_by_id(ids, boxes))
    b.close()
