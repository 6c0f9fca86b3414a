"""The N>1 path of bench.py on CPU: two gloo ranks, barrier, max-over-ranks
timing and the whole-job (weak-scaling) aggregate; the reference arm runs on
rank 0 only."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    w, r, l = bench.dist_env()
    dist = bench.dist_setup(w, "gloo")
    bench.barrier(dist)
    t = bench.reduce_max(dist, 1.0 + r)          # rank r "took" 1+r seconds
    v = bench.whole_job_value(w, cells=1000, steps=10, max_seconds=t)
    ref = bench.run_reference(None, w, r, l) if r != 0 else "rank0"
    q.put((r, t, v, ref))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, t, v, ref in out:
        assert t == 2.0                      # max over ranks
        assert v == 2 * 1000 * 10 / 2.0      # all replicas' cells / slowest rank
    assert out[1][3] is None                 # reference arm: rank 1 does no work


def test_single_rank_defaults():
    os.environ.pop("WORLD_SIZE", None)
    w, r, l = bench.dist_env()
    assert (w, r) == (1, 0)
    assert bench.dist_setup(1, "gloo") is None
    assert bench.reduce_max(None, 3.5) == 3.5
