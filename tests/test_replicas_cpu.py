"""Replicas (bench.py --gpus N): the ranks share no data path; the timing is bracketed by barriers and reduced with
MAX over ranks, and the whole-job value counts the units of every rank. Run here as two gloo ranks on the CPU."""
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


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        ms = bench.reduce_max(10.0 + rank, world)          # rank 1 is the slowest
        units = 1000 * world                                # weak scaling: every rank its own replica
        q.put((rank, ms, units / (ms / 1e3)))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [11.0, 11.0]
    assert got[0][2] == pytest.approx(2000 / 0.011)
