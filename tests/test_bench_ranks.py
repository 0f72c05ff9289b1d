"""The multi-rank logic of bench.py on CPU: two gloo ranks each take their own
pose slice (no overlap, nothing left out) and agree on the slowest rank's
time, which sets the whole-job throughput."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dofs = np.arange(10 * world * 6, dtype=np.float32).reshape(-1, 6)
        mine = bench.shard(dofs, world, rank)
        slow = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world, device="cpu")
        q.put((rank, mine[:, 0].tolist(), slow))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in procs:
        r, first_col, slow = q.get(timeout=120)
        got[r] = (first_col, slow)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rows0, rows1 = np.array(got[0][0]) / 6, np.array(got[1][0]) / 6
    assert len(rows0) == len(rows1) == 10
    assert sorted(np.concatenate([rows0, rows1]).tolist()) == list(range(20))
    assert got[0][1] == got[1][1] == [2.0, 5.0]


def test_one_rank_is_the_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    d = np.zeros((7, 6), np.float32)
    assert bench.shard(d, 1, 0).shape == (7, 6)
    assert bench.max_over_ranks([3.0], 1) == [3.0]
