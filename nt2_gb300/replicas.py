"""Replica bookkeeping for runs on several GPUs (one process per GPU).

Every configuration of the evaluator is independent per option, element or
stream, so several GPUs run replicas: each rank evaluates its own batch (weak
scaling) or its own contiguous shard of one batch (strong scaling), with no
exchange on the data path.  The only collectives are the barrier around a
timed region and the maximum of the ranks' times, which give the whole job's
throughput.  Works with the nccl backend (CUDA tensors) and gloo (CPU).
"""
from __future__ import annotations

import os


def env():
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous [begin, end) of n units owned by `rank`; shards differ by at most one unit
    and cover [0, n) exactly."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    q, r = divmod(n, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def _device():
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    """The largest value any rank holds (the job's time is its slowest rank's)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, world: int, seconds_max: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world / seconds_max
