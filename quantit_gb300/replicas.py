"""Multi-GPU runs: independent replicas, one solve per GPU (the DMRG sweep is
sequential bond after bond, so a solve does not shard; independent solves do).

No collective touches the data path.  The only cross-rank traffic is the timing
reduction at the end of a measurement: the maximum of every rank's time, and
the number of units (sweeps, solves) all ranks processed.
"""
import os


def env():
    """(rank, world size, local rank) from the torchrun environment (1 process if unset)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def replica_seed(base, rank):
    """Seed of rank's replica: every replica solves its own random start."""
    return int(base) * 1000003 + int(rank)


def _reduce(values, op):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return [float(x) for x in t.cpu()]


def max_over_ranks(values):
    import torch.distributed as dist
    return _reduce(values, dist.ReduceOp.MAX)


def sum_over_ranks(values):
    import torch.distributed as dist
    return _reduce(values, dist.ReduceOp.SUM)


def whole_job_time_per_unit(seconds, units):
    """Seconds per unit of the whole job: the slowest rank's time over the units
    all ranks processed (weak scaling: every rank processes its own units)."""
    t = max_over_ranks([seconds])[0]
    n = sum_over_ranks([units])[0]
    return t / n if n > 0 else float("nan"), t, n
