"""bench.py's multi-rank plumbing on the CPU (gloo, world size 2): the path
runs as independent replica streams per rank, so the only cross-rank steps are
the barrier around the timed region and the max-over-ranks of the elapsed
time; the reference arm prints from rank 0 only."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier(ws)
    elapsed = 10.0 + 5.0 * rank  # rank 1 is the slow one
    worst = bench.reduce_max(elapsed, ws)
    Path(out_dir, f"rank{rank}.txt").write_text(f"{worst}")
    bench.barrier(ws)
    dist.destroy_process_group()


def test_two_rank_max_and_barrier(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    assert Path(tmp_path, "rank0.txt").read_text() == "15.0"
    assert Path(tmp_path, "rank1.txt").read_text() == "15.0"


def test_reference_arm_silent_on_other_ranks(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup = 1, 3

    bench.run_reference(A())
    assert capsys.readouterr().out == ""
