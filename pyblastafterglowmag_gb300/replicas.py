"""Replica execution over ranks: one process per GPU, no exchange on the data path.

Blastwaves are independent (the reference evolves each (layer, shock) pair on
its own; the only shared objects are the read-only grids and kernel tables),
so a job of many blastwaves or parameter sets splits into contiguous shards,
one per rank, each run as its own batch on its own GPU. The ranks talk on the
host only: a barrier around a timed region, the slowest rank's time, and the
sum of the work units. These helpers hold that logic so that it is the same in
the benchmark and in the multi-process tests (gloo on CPU).
"""
import os


def dist_info():
    """(rank, world_size, local_rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init(world, backend="gloo"):
    """Join the process group when there is more than one rank (host-side
    collectives only: gloo needs no GPU)."""
    if world <= 1:
        return
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)


def shard(n, rank, world):
    """The contiguous block of n items that rank `rank` of `world` owns: sizes
    differ by at most one, every item is owned exactly once, in order."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError(f"bad shard request n={n} rank={rank} world={world}")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return range(lo, lo + q + (1 if rank < r else 0))


def barrier(world, device=None):
    """Device synchronisation, then a host barrier across ranks."""
    if device is not None:
        import torch
        torch.cuda.synchronize(device)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(x, world, op):
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world):
    """The largest value over ranks (the slowest rank's time)."""
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.MAX if world > 1 else None)


def sum_over_ranks(x, world):
    """The sum over ranks (the job's work units)."""
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.SUM if world > 1 else None)


def job_rate(units, seconds, world):
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    total = sum_over_ranks(units, world)
    t = max_over_ranks(seconds, world)
    return total / t if t > 0 else float("nan")
