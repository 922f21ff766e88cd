"""The multi-GPU path is replicas only (no data-path collective): each rank
evaluates its own shard and the job's time is the slowest rank's.  This runs
that host logic with world size 2 over gloo on the CPU; each rank prices its
shard of one Black-Scholes batch with the oracle, and rank 0 checks that the
gathered shards equal the whole batch and that the time aggregate is the max."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from nt2_gb300 import replicas


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("n,world", [(10, 3), (7, 2), (1, 4), (0, 2), (1 << 20, 8)])
def test_shards_cover_exactly(n, world):
    seen = []
    for r in range(world):
        b, e = replicas.shard(n, world, r)
        assert 0 <= b <= e <= n
        seen.extend(range(b, e))
    assert seen == list(range(n))
    sizes = [replicas.shard(n, world, r)[1] - replicas.shard(n, world, r)[0] for r in range(world)]
    assert max(sizes) - min(sizes) <= 1


def _rank(rank, world, port, n, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import oracle_lib
    rng = np.random.default_rng(0)
    S = rng.uniform(5, 30, n).astype(np.float32)
    K = rng.uniform(1, 100, n).astype(np.float32)
    T = rng.uniform(0.25, 10, n).astype(np.float32)
    b, e = replicas.shard(n, world, rank)
    call, put = oracle_lib.bs(S[b:e].copy(), K[b:e].copy(), T[b:e].copy(), 0.02, 0.30, threads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (b, e, call, put))
    t = replicas.max_over_ranks(float(rank + 1) * 0.5, world)
    replicas.barrier(world)
    if rank == 0:
        rc, rp = oracle_lib.bs(S, K, T, 0.02, 0.30, threads=1)
        whole_c = np.concatenate([p[2] for p in sorted(parts, key=lambda p: p[0])])
        whole_p = np.concatenate([p[3] for p in sorted(parts, key=lambda p: p[0])])
        out.put((bool(np.array_equal(whole_c.view(np.uint32), rc.view(np.uint32)) and
                      np.array_equal(whole_p.view(np.uint32), rp.view(np.uint32))), t,
                 replicas.job_throughput(n // world, world, t)))
    dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, n = 2, 10007
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    equal, tmax, thr = q.get(timeout=10)
    assert equal
    assert tmax == 1.0                        # max over ranks of 0.5 and 1.0
    assert thr == (n // world) * world / 1.0
