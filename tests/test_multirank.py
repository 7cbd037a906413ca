"""CPU tests of bench.py's multi-rank path (world size 2, gloo, 127.0.0.1).

bench.py --gpus N runs one independent replica per rank: a barrier on both
sides of the timed region, the slowest rank's time reported, and the
reference arm on rank 0 only.  The host logic is checked here without a GPU."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import sys
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = bench.dist_env()
        bench.rank_barrier(w)
        # each rank reports its own time; everyone gets the slowest one
        mx = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")
        bench.rank_barrier(w)
        out.put((r, w, lr, mx))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, w, lr) for r, w, lr, _ in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(mx == 15.0 for *_, mx in res)


def test_single_process_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    bench.rank_barrier(1)


def test_reference_arm_runs_on_rank0_only(capsys, monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 1, 0, 2
    bench.run_reference(A())
    assert capsys.readouterr().out == ""
