"""Replica bookkeeping for runs over several GPUs.

The batch evaluation has no exchange step: every rank evaluates its own
independent batch of structures (its own seed), so a multi-GPU run is a set
of replicas.  The whole-job throughput is the work of all ranks divided by
the time of the slowest one.
"""
import torch
import torch.distributed as dist


def replica_seed(seed, rank):
    """Seed of the batch generated on ``rank``."""
    return int(seed) + 1000 * int(rank)


def _group_size():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def _reduce(x, op, device):
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if _group_size() > 1:
        dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, device=None):
    return _reduce(x, dist.ReduceOp.MAX, device)


def sum_over_ranks(x, device=None):
    return _reduce(x, dist.ReduceOp.SUM, device)


def job_rate(units, seconds, device=None):
    """Units processed by all ranks per second of the slowest rank."""
    return sum_over_ranks(units, device) / max_over_ranks(seconds, device)
