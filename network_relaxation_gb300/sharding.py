"""Multi-GPU layout of batched relaxation: one process per GPU, each rank
relaxes its own independent batch of networks (the batch is the unit of
work; networks never span ranks), so the data path has no collective.  The
only cross-rank step is reducing the timing (max over ranks) and the
network counts (sum), which works on any torch.distributed backend (nccl on
GPUs, gloo in the CPU tests).
"""
import os

from . import workloads


def rank_info():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_c4_params(rank, n=workloads.C4_COUNT):
    """The uneven-batch parameters of one rank: rank r uses generator seeds
    C4_SEED + n*r .. C4_SEED + n*r + n - 1, so ranks never share a network
    and rank 0 is the single-GPU workload."""
    return workloads.c4_params(n=n, seed=workloads.C4_SEED + n * rank)


def reduce_timing(dist, ms, n_networks, device=None):
    """Max of the per-rank step time and sum of relaxed networks over ranks.
    Returns (max_ms, total_networks); identity when dist is None."""
    if dist is None:
        return ms, n_networks
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(n_networks)], dtype=torch.float64, device=device)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), int(c.item())
