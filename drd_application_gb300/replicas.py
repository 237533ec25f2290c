"""Replicas-only multi-GPU aggregation.

A grid of the reference's sizes (at most a few million cells) is solved on one GPU, and the
time steps of one run depend on each other, so the path does not shard: N ranks run N
independent replicas (different seeds), with no collective on the data path.  The only
communication is this aggregation of the timings: throughput = steps of all ranks divided by
the slowest rank's elapsed time.
"""


def replica_throughput(local_steps, local_seconds, dist=None, device="cpu"):
    """(total steps / max seconds over ranks, max seconds).  `dist` is torch.distributed (or
    None for one process); tensors live on `device` (cpu for gloo, cuda for nccl)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return local_steps / local_seconds, local_seconds
    import torch

    steps = torch.tensor([float(local_steps)], dtype=torch.float64, device=device)
    secs = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(steps, op=dist.ReduceOp.SUM)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX)
    return float(steps.item()) / float(secs.item()), float(secs.item())


def replica_seed(rank, base=0):
    """Seed of the workload replica a rank runs."""
    return base + rank
