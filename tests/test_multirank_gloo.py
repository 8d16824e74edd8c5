"""The multi-rank host logic on CPU with gloo, world size 2: the max-over-ranks timing reduction of
bench.py, the reference arm under torchrun (rank 0 alone measures and prints one line, the other
rank exits 0 without work), and the sharding of one batch (parry_gb300.sharding): contiguous ray
ranges and cost-balanced pair ranges, each rank's range run through the oracle on its CPU rank, and
the results gathered to rank 0 in input order equal the single-rank answer."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.reduce_max(1.5 + rank, world)
    Path(out_dir, f"rank{rank}.txt").write_text(repr(got))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    assert [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)] == [2.5, 2.5]


def test_reduce_max_alone_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_max(3.25, 1) == 3.25


def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup",
           "0", "--n-rays", "20000"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0


def _shard_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    from parry_gb300 import sharding as S
    from parry_gb300 import workloads as W
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rays: one batch of 3,001 rays over a small terrain, contiguous ranges
    v, i = W.terrain_mesh(32, 16, seed=4)
    rays = W.terrain_rays(3001, 32, 16, seed=4)
    a, b = S.ray_ranges(len(rays), world)[rank]
    f, t, n = O.TriMesh(v, i).cast_rays_and_get_normal(rays[a:b], 100.0, threads=1)
    got_rays = S.gather({"feature": f, "toi": t, "normal": n}, rank, world)
    # pairs: uneven hull pairs, ranges balanced by support cost
    s, pairs = W.hull_pairs(1500, seed=9)
    types, params, _, _ = s.arrays()
    cost = S.support_cost(types, params, pairs)
    a, b = S.pair_ranges(cost, world)[rank]
    h, o, _ = O.contacts(s, pairs[a:b], 0.0, threads=1)
    got_pairs = S.gather({"has": h, "out": o}, rank, world)
    if rank == 0:
        np.savez(Path(out_dir, "gathered.npz"), **{"ray_" + k: v for k, v in got_rays.items()},
                 **{"pair_" + k: v for k, v in got_pairs.items()})
    else:
        assert got_rays is None and got_pairs is None
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_batch_gathers_to_the_single_rank_answer(tmp_path):
    import numpy as np
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    from parry_gb300 import workloads as W
    port = _free_port()
    mp.start_processes(_shard_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    g = np.load(tmp_path / "gathered.npz")
    v, i = W.terrain_mesh(32, 16, seed=4)
    rays = W.terrain_rays(3001, 32, 16, seed=4)
    f, t, n = O.TriMesh(v, i).cast_rays_and_get_normal(rays, 100.0, threads=1)
    np.testing.assert_array_equal(g["ray_feature"], f)
    np.testing.assert_array_equal(g["ray_toi"], t)
    np.testing.assert_array_equal(g["ray_normal"], n)
    s, pairs = W.hull_pairs(1500, seed=9)
    h, o, _ = O.contacts(s, pairs, 0.0, threads=1)
    np.testing.assert_array_equal(g["pair_has"], h)
    np.testing.assert_array_equal(g["pair_out"], o)


def test_shard_ranges():
    import numpy as np
    sys.path.insert(0, str(ROOT))
    from parry_gb300 import sharding as S
    for n, w in ((10, 3), (3, 4), (0, 2), (1 << 20, 8)):
        r = S.ray_ranges(n, w)
        assert r[0][0] == 0 and r[-1][1] == n and all(r[k][1] == r[k + 1][0] for k in range(w - 1))
        sizes = [e - s for s, e in r]
        assert max(sizes) - min(sizes) <= 1
    rng = np.random.default_rng(2)
    cost = rng.integers(2, 513, 100_000)
    for w in (1, 2, 3, 8):
        r = S.pair_ranges(cost, w)
        assert r[0][0] == 0 and r[-1][1] == len(cost) and all(r[k][1] == r[k + 1][0] for k in range(w - 1))
        shares = [int(cost[s:e].sum()) for s, e in r]
        assert max(shares) - min(shares) <= 2 * int(cost.max())
    # sorted costs (the pairs binned by cost): the cheap half takes many more pairs than the dear one
    r = S.pair_ranges(np.sort(cost), 2)
    assert r[0][1] - r[0][0] > r[1][1] - r[1][0]
    assert S.pair_ranges(np.zeros(0, np.int64), 3) == [(0, 0)] * 3
