"""Multi-process (world_size 2 and 4, gloo, CPU) tests of the batch
sharding and the timing reduction used by bench.py under torchrun, and of a
rank leaving between steps (the others learn of it at their next
reduction, as an error)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from network_relaxation_gb300 import sharding

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = sharding.rank_info()
    params = sharding.rank_c4_params(r, n=8)
    seeds = [q["seed"] for q in params]
    ms, total = sharding.reduce_timing(dist, 10.0 * (r + 1), len(params))
    out[r] = (r, w, lr, seeds, ms, total)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_rank_sharding_and_reduction(world):
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    res = [out[r] for r in range(world)]
    assert [r[:3] for r in res] == [(r, world, r) for r in range(world)]
    # disjoint seeds, rank 0 is the single-GPU workload
    seeds = [set(r[3]) for r in res]
    assert sum(len(x) for x in seeds) == len(set().union(*seeds)) == 8 * world
    from network_relaxation_gb300 import workloads

    assert res[0][3] == [q["seed"] for q in workloads.c4_params(n=8)]
    # max over ranks of the step time, sum of the networks
    assert all(r[4] == 10.0 * world and r[5] == 8 * world for r in res)


def _worker_leaves(rank, world, port, out):
    """Rank 1 leaves between steps (nothing in flight); rank 0's next
    reduction must end with an error, not wait forever."""
    import datetime

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from network_relaxation_gb300 import sharding

    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    sharding.reduce_timing(dist, 1.0, 1)  # one step together
    if rank == 1:
        out[1] = "left"
        os._exit(0)
    try:
        sharding.reduce_timing(dist, 2.0, 1)
        out[0] = "no error"
    except Exception as e:  # gloo reports the lost peer or the timeout
        out[0] = "error " + type(e).__name__


def test_rank_that_leaves_is_detected_by_the_next_reduction():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker_leaves, args=(2, port, out), nprocs=2, join=True)
    assert out[1] == "left"
    assert out[0].startswith("error"), out[0]


def test_single_process_reduction_is_identity():
    from network_relaxation_gb300 import sharding

    assert sharding.reduce_timing(None, 3.5, 7) == (3.5, 7)


def _worker_split(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from network_relaxation_gb300 import sharding

    dist.init_process_group("gloo", rank=rank, world_size=world)
    idx, params = sharding.split_c4_params(rank, world)
    # each rank "relaxes" its share: reports carry the index and the seed
    vals = [(float(i), float(q["seed"])) for i, q in zip(idx, params)]
    rows = sharding.gather_reports(dist, idx, vals, 512, 2)
    cost = sum(sharding.expected_cost(q) for q in params)
    out[rank] = (idx, rows, cost, max(sharding.expected_cost(q) for q in params))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_one_batch_split_across_ranks_covers_every_network_once_and_balances(world):
    """Split mode: ONE 512-network batch partitioned by LPT on expected cost;
    every network on exactly one rank, the reports gathered in batch order on
    every rank, and the predicted loads within one network's cost of each
    other (the LPT bound)."""
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker_split, args=(world, port, out), nprocs=world, join=True)
    res = [out[r] for r in range(world)]
    all_idx = sorted(i for r in res for i in r[0])
    assert all_idx == list(range(512))
    from network_relaxation_gb300 import workloads

    seeds = [q["seed"] for q in workloads.c4_params()]
    for r in res:
        assert [row[0] for row in r[1]] == [float(i) for i in range(512)]
        assert [row[1] for row in r[1]] == [float(s) for s in seeds]
    loads = [r[2] for r in res]
    assert max(loads) - min(loads) <= max(r[3] for r in res)


def test_lpt_split_balances_the_oracle_step_counts():
    """The expected-cost model ranks the uneven batch well enough that the
    split's TRUE FP64 work (the oracle's step counts x N) is balanced: the
    largest rank within 5 % (2 ranks) / 15 % (4 ranks) / 30 % (8 ranks) of the
    mean."""
    import json

    from network_relaxation_gb300 import sharding, workloads

    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "c4_oracle.json")))["networks"]
    true = [r["steps"] * r["n_points"] for r in golden]
    params = workloads.c4_params()
    assert [q["seed"] for q in params] == [r["seed"] for r in golden]
    for world, bound in ((2, 1.05), (4, 1.15), (8, 1.30)):
        parts = sharding.lpt_partition([sharding.expected_cost(q) for q in params], world)
        assert sorted(i for p in parts for i in p) == list(range(512))
        loads = [sum(true[i] for i in p) for p in parts]
        assert max(loads) <= bound * sum(loads) / world, (world, loads)
    assert sharding.lpt_partition([5.0, 1.0, 1.0, 3.0], 2) == [[0], [1, 2, 3]]
    assert sharding.gather_reports(None, [2, 0], [(1.0,), (2.0,)], 3, 1) == [(2.0,), None, (1.0,)]
