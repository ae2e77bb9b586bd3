"""Replica runs on several GPUs of one node.

A SENSE / FISTA solve is not sharded here: each rank runs an independent replica
(its own plan, data and solve) and the job's throughput is the work of all ranks
divided by the slowest rank's time.  The only cross-rank traffic is this
bookkeeping, never the data path.
"""
import torch
import torch.distributed as dist


def world():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def max_over_ranks(x, device=None):
    """Maximum of a float over all ranks (itself when not distributed)."""
    if world() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, seconds_local, device=None):
    """(units of all ranks) / (max over ranks of the timed seconds), and that max."""
    s = max_over_ranks(seconds_local, device)
    return world() * units_per_rank / s, s
