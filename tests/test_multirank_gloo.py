"""The multi-rank host logic of bench.py on CPU with gloo, world size 2: the max-over-ranks timing
reduction, and the reference arm under torchrun (rank 0 alone measures and prints one line, the
other rank exits 0 without work). The path itself shards as independent replicas (no collective on
the data path), so these are the only cross-rank steps."""
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
