"""Shared test helpers: a structural validator for BvhNodeWide arrays and header parsing."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def header_symbols() -> list[str]:
    """Every function declared in include/*.h."""
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(parrygpu_\w+)\s*\(", txt)
    return sorted(set(names))


def _node(w: np.ndarray, side: int):
    u = w.view(np.uint32)
    o = 8 * side
    return w[o:o + 3], int(u[o + 3]), w[o + 4:o + 7], int(u[o + 7])


def assert_well_formed(nodes: np.ndarray, n_leaves: int, leaf_data_is_index: bool = True) -> None:
    """Restatement of Bvh::assert_well_formed (src/partitioning/bvh/bvh_validation.rs:61-141) on a
    (wide_nodes, 16) float32 array in BvhNodeWide layout: no loops, leaf counts add up, every
    parent AABB contains its children, and every leaf index appears exactly once."""
    if n_leaves == 0:
        assert len(nodes) == 0
        return
    lc = lambda d: d & 0x3FFFFFFF
    if n_leaves == 1:
        mn, ch, mx, d = _node(nodes[0], 0)
        _, _, _, d2 = _node(nodes[0], 1)
        assert lc(d) == 1 and lc(d2) == 0
        return
    seen_nodes = set()
    seen_leaves = []
    stack = [0]
    while stack:
        i = stack.pop()
        assert i not in seen_nodes, f"loop: node {i} visited twice"
        seen_nodes.add(i)
        for side in (0, 1):
            mn, ch, mx, d = _node(nodes[i], side)
            assert np.all(mn <= mx), f"inverted AABB in node {i}.{side}"
            if lc(d) == 1:
                seen_leaves.append(ch)
            else:
                c = nodes[ch]
                cmn0, _, cmx0, cd0 = _node(c, 0)
                cmn1, _, cmx1, cd1 = _node(c, 1)
                assert np.all(mn <= cmn0) and np.all(mx >= cmx0), f"node {i}.{side} does not contain its left child"
                assert np.all(mn <= cmn1) and np.all(mx >= cmx1), f"node {i}.{side} does not contain its right child"
                assert lc(d) == lc(cd0) + lc(cd1), f"leaf count mismatch at {i}.{side}"
                stack.append(ch)
    assert len(seen_nodes) == len(nodes), "unreachable wide nodes"
    assert len(seen_leaves) == n_leaves
    if leaf_data_is_index:
        assert sorted(seen_leaves) == list(range(n_leaves))


def brute_force_pairs(aabbs: np.ndarray) -> np.ndarray:
    """All (i < j) with intersecting AABBs (inclusive), sorted; O(n^2 / block) numpy."""
    n = len(aabbs)
    mn, mx = aabbs[:, :3], aabbs[:, 3:]
    out = []
    for s in range(0, n, 512):
        e = min(n, s + 512)
        ok = np.all(mn[s:e, None, :] <= mx[None, :, :], axis=-1) & np.all(mx[s:e, None, :] >= mn[None, :, :], axis=-1)
        ii, jj = np.nonzero(ok)
        ii = ii + s
        keep = ii < jj
        out.append(np.stack([ii[keep], jj[keep]], axis=1))
    p = np.concatenate(out).astype(np.uint32) if out else np.zeros((0, 2), np.uint32)
    order = np.lexsort((p[:, 1], p[:, 0]))
    return p[order]


def random_aabbs(n: int, seed: int, extent: float = 100.0, size: float = 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.uniform(-extent, extent, size=(n, 3))
    h = rng.uniform(0.05, size, size=(n, 3))
    return np.concatenate([c - h, c + h], axis=1).astype(np.float32)


def serialized_links(nodes: np.ndarray) -> tuple[np.ndarray, dict]:
    """The `parents` and `leaf_node_indices` a parry Bvh keeps beside its nodes (bvh_tree.rs:1755-1761)
    recomputed from the nodes alone: parents[w] = BvhNodeIndex (wide << 1 | is_right) of the slot
    holding wide node w (0 for the root); leaf index -> BvhNodeIndex of its slot."""
    parents = np.zeros(len(nodes), np.uint64)
    leaves = {}
    u = nodes.view(np.uint32)
    for w in range(len(nodes)):
        for side in (0, 1):
            ch, d = int(u[w, 8 * side + 3]), int(u[w, 8 * side + 7]) & 0x3FFFFFFF
            if d == 1:
                leaves[ch] = (w << 1) | side
            elif d > 1:
                parents[ch] = (w << 1) | side
    return parents, leaves
