"""bench.py's multi-process host logic on CPU: world size 2 over gloo (no GPU).

Each rank is an independent replica; the process group carries only the barrier and the
maximum of the ranks' timed regions, which rank 0 reports."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    r, local, w, dist = bench.dist_setup(world, backend="gloo")
    assert (r, local, w) == (rank, rank, world)
    bench.barrier(dist)
    out[rank] = bench.max_over_ranks(times[rank], dist)
    bench.barrier(dist)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_max_over_ranks_world_size_2():
    world, times = 2, [0.25, 0.75]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert dict(out) == {0: 0.75, 1: 0.75}


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        rank, local, world, dist = bench.dist_setup(1)
        assert (rank, local, world, dist) == (0, 0, 1, None)
        assert bench.max_over_ranks(1.5, None) == 1.5
    finally:
        os.environ.update(env)
