"""The N>1 bench path on CPU: two gloo ranks run bench.py's replica plumbing
(barrier, max-over-ranks of the timed region, sum of processed queries), the
same code the torchrun launch uses on GPUs."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist()
    d.barrier()
    t = d.max(1.0 + rank)          # slowest rank's time
    n = d.sum(1000.0 * (rank + 1))  # queries processed by all ranks
    out.put((rank, t, n, d.world))
    d.pg.destroy_process_group()


def test_two_rank_max_and_sum():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n, world in res:
        assert world == 2 and t == 2.0 and n == 3000.0
