"""The multi-rank host path of bench.py on CPU (gloo, world_size 2): independent
right-hand sides shard across ranks with no data-path collective, and the step time is
the maximum over ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "gdmr-solver_gb300"))
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import problems
    import bench
    seeds = problems.shard_seeds(4, rank)
    gathered = [None] * world
    dist.all_gather_object(gathered, seeds)
    t = bench.max_over_ranks(1.0 + rank, world)
    bench.barrier(world)
    out.put((rank, gathered, t))
    dist.destroy_process_group()


def test_two_ranks_shard_disjoint_and_take_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, t in res:
        assert t == 2.0                      # max over ranks
        a, b = gathered
        assert len(a) == len(b) == 4 and not set(a) & set(b)
