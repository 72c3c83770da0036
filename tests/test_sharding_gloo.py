"""The multi-rank host path of bench.py on CPU (gloo, world_size 2): independent
right-hand sides shard across ranks with no data-path collective, and the step time is
the maximum over ranks.  In the second test every rank really solves its shard (bench.py's
own workload builder at a 12^3 grid; the host oracle stands in for the GPU, which this
machine does not have) and the ranks' answers are gathered and checked against a sparse
direct solve: each right-hand side is solved once, by one rank, to the tolerance."""
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


def _solve_worker(rank, world, port, out):
    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "gdmr-solver_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import time
    import bench
    import oracle
    import problems
    shape = (12, 12, 12)
    A, B = bench.build_workload(3, rank, shape)           # this rank's shard of right-hand sides
    seeds = problems.shard_seeds(3, rank)
    o = oracle.Oracle(A, 24, 8, threads=1, fuse_deflation=True)
    bench.barrier(world)
    t = time.perf_counter()
    X = [o.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=500)["x"] for i, b in enumerate(B)]
    el = bench.max_over_ranks(time.perf_counter() - t, world)
    bench.barrier(world)
    mine = [(sd, b, x) for sd, b, x in zip(seeds, B, X)]
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    out.put((rank, gathered, el))
    dist.destroy_process_group()


def test_two_ranks_solve_their_shards_and_gather_correct_answers():
    import numpy as np
    import scipy.sparse.linalg as spl
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "gdmr-solver_gb300"))
    import problems
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_solve_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    A = problems.helmholtz((12, 12, 12), 24.0, 0.1).to_scipy().tocsc()
    lu = spl.splu(A)
    for rank, gathered, el in res:
        assert el > 0
        items = [it for part in gathered for it in part]
        seeds = [sd for sd, _, _ in items]
        assert sorted(seeds) == sorted(problems.shard_seeds(3, 0) + problems.shard_seeds(3, 1))
        for sd, b, x in items:
            assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1e-10
            ref = lu.solve(b)
            assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-8
    assert res[0][2] == res[1][2]               # both ranks report the same (max) time
