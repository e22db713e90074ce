"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): the path
runs replicas only (no data exchange between ranks), so the only cross-rank
logic is the timing aggregation -- whole-job units summed over ranks divided
by the slowest rank's time -- and the barrier around the timed region."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    import sys
    import pathlib
    root = pathlib.Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local = bench.dist_env()
    bench.dist_init(w, "gloo")
    bench.barrier(w)
    # rank r "processed" 100*(r+1) cells in (r+1) seconds
    value, tmax = bench.aggregate(float(r + 1), 100.0 * (r + 1), w)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, value, tmax))


def test_aggregate_two_ranks_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, value, tmax in out:
        assert tmax == pytest.approx(2.0)
        assert value == pytest.approx((100.0 + 200.0) / 2.0)


def test_single_rank_aggregate_is_plain_ratio():
    import sys
    import pathlib
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parents[1]))
    import bench
    assert bench.aggregate(2.0, 10.0, 1) == (5.0, 2.0)
