"""Sharding one batch of independent queries over the ranks of a job (one process per GPU).

parry's queries are pure functions of their inputs (`QueryDispatcher: Send + Sync`,
src/query/query_dispatcher.rs:408), so a batch splits without any exchange of data between ranks:

- rays (TriMesh / shape-set ray casts): every rank holds a replica of the mesh and its BVH (about
  17 MB at most) and casts a contiguous range of the rays;
- pairs (query::contact, contact manifolds, shape casts): every rank holds the shapes and takes a
  contiguous range of the pair list, the ranges cut where the running support-scan cost (vertices a
  support evaluation scans, the key the library bins pairs by) reaches an equal share, so that a rank
  with the 256-vertex hulls does not get as many pairs as one with balls;
- results come back to the host and are concatenated in rank order, which is input order. No GPU
  reads another GPU's memory: the gather moves host arrays through the process group.

The functions here are the host logic only; each rank runs its range through the library on its
own device (see bench.py), and tests run them over gloo on CPU.
"""
from __future__ import annotations

import numpy as np


def ray_ranges(n: int, world: int) -> list[tuple[int, int]]:
    """[start, end) of each rank's rays: contiguous, sizes differing by at most one."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(int(n), world)
    out, start = [], 0
    for r in range(world):
        end = start + base + (1 if r < extra else 0)
        out.append((start, end))
        start = end
    return out


def support_cost(types: np.ndarray, params: np.ndarray, pairs: np.ndarray) -> np.ndarray:
    """Per pair: the vertices one support evaluation of the pair scans (a convex polyhedron's or a
    triangle's vertex count, 1 for a ball, cuboid or capsule, summed over the two shapes); the key
    the contact kernels bin pairs by."""
    from .shapes import CONVEX, TRIANGLE
    t = np.asarray(types, np.uint32)
    counts = np.asarray(params, np.float32).reshape(-1, 4).view(np.uint32)[:, 1]
    per_shape = np.where((t == CONVEX) | (t == TRIANGLE), np.minimum(counts, 1023), 1).astype(np.int64)
    p = np.asarray(pairs, np.int64).reshape(-1, 2)
    return per_shape[p[:, 0]] + per_shape[p[:, 1]]


def pair_ranges(cost: np.ndarray, world: int) -> list[tuple[int, int]]:
    """[start, end) of each rank's pairs: contiguous, cut where the running cost reaches r / world of
    the total (each cut at the first pair whose running cost reaches the share)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    cost = np.asarray(cost, np.int64)
    n = len(cost)
    if n == 0:
        return [(0, 0)] * world
    run = np.cumsum(cost)
    total = int(run[-1])
    cuts = [0]
    for r in range(1, world):
        cuts.append(max(cuts[-1], int(np.searchsorted(run, (total * r + world - 1) // world, side="left")) + 1))
    cuts = [min(c, n) for c in cuts] + [n]
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def gather(local: dict, rank: int, world: int, group=None) -> dict | None:
    """Concatenates each rank's result arrays in rank order on rank 0 (host arrays through the
    process group; other ranks get None). With world == 1 the local result is returned."""
    if world == 1:
        return local
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local, parts, dst=0, group=group)
    if rank != 0:
        return None
    return {k: np.concatenate([p[k] for p in parts]) for k in local}
