"""Multi-GPU layout of batched relaxation: one process per GPU; networks
never span ranks, so the data path has no collective.  Two layouts:

  weak   every rank relaxes its own independent batch (rank_c4_params);
  split  ONE batch is partitioned across the ranks by network
         (split_c4_params): longest-processing-time-first on each network's
         expected cost, N x expected FIRE iterations, so the ranks finish
         together.

The only cross-rank steps are reducing the timing (max over ranks) and the
network counts (sum), and gathering the per-network reports at the end,
which work on any torch.distributed backend (nccl on GPUs, gloo in the CPU
tests).
"""
import math
import os

from . import workloads

# ln(expected FIRE iterations to max|F| < 1e-10) of a diluted triangular
# lattice, linear in (1, ln L, p, log10 kappa, ln(gamma + 1e-3)): a least-
# squares fit to the FP64 oracle's step counts on the 512 networks of the
# uneven batch (correlation 0.96 in log space).  Only its ranking matters:
# it balances work across ranks; the relaxation itself never reads it.
_ITER_FIT = (11.5086, 0.90467, -11.7228, -0.88660, 0.086088)


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


def expected_iterations(n_points, p, kappa, gamma):
    """Expected FIRE iterations of a diluted lattice of n_points nodes with
    bond probability p, bending stiffness kappa, at shear gamma (the fit
    above; L = sqrt(n_points))."""
    c = _ITER_FIT
    L = math.sqrt(max(1, n_points))
    return math.exp(c[0] + c[1] * math.log(L) + c[2] * p + c[3] * math.log10(kappa) + c[4] * math.log(gamma + 1e-3))


def expected_cost(q):
    """N x expected iterations of one network of the uneven batch."""
    n = q["L"] * q["L"]
    return n * expected_iterations(n, q["p"], q["kappa"], q["gamma"])


def lpt_partition(costs, world):
    """Longest-processing-time-first: items by decreasing cost (ties by
    index), each to the rank with the smallest load so far (ties: the lowest
    rank).  Returns world lists of item indices, each in increasing order.
    Every item lands on exactly one rank, and the largest load exceeds the
    smallest by at most the largest single cost."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += costs[i]
        parts[r].append(i)
    return [sorted(p) for p in parts]


def split_c4_params(rank, world, n=workloads.C4_COUNT):
    """Rank `rank`'s share of ONE uneven batch split across `world` ranks:
    (indices into the batch, their parameters)."""
    params = workloads.c4_params(n=n)
    parts = lpt_partition([expected_cost(q) for q in params], world)
    idx = parts[rank]
    return idx, [params[i] for i in idx]


def gather_reports(dist, idx, values, n_total, width, device=None):
    """Collects per-network values (one tuple of `width` floats per index in
    idx) from every rank into one list of n_total entries in batch order, on
    every rank (`width` is passed, not inferred, so a rank with no networks
    still joins the same collective).  Identity layout when dist is None."""
    if dist is None:
        out = [None] * n_total
        for i, v in zip(idx, values):
            out[i] = tuple(v)
        return out
    import torch

    t = torch.zeros((n_total, width + 1), dtype=torch.float64, device=device)
    for i, v in zip(idx, values):
        t[i, 0] = 1.0
        t[i, 1:] = torch.tensor(v, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if not bool((t[:, 0] == 1.0).all()):
        raise RuntimeError("gather_reports: a network was reported by no rank or by several")
    return [tuple(float(x) for x in row[1:]) for row in t.cpu()]
