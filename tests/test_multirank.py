"""bench.py's N-replica logic on two CPU ranks (gloo): each rank renders its
own frames (no exchange), and the job's numbers are the slowest rank's time
and the sum of all ranks' rays."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    ms, rays = bench.reduce_over_ranks(dist, 10.0 * (rank + 1), 1000.0 * (rank + 1), device="cpu")
    out.put((r, w, local, ms, rays))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_reduce_max_time_and_sum_rays():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, w, local) for r, w, local, _, _ in results] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, ms, rays in results:
        assert ms == 20.0 and rays == 3000.0


def test_one_rank_passes_through():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_over_ranks(None, 5.0, 7.0) == (5.0, 7.0)
