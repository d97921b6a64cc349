"""Multi-process (world_size 2, gloo, CPU) test of the batch sharding and
the timing reduction used by bench.py under torchrun."""
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


def test_two_rank_sharding_and_reduction():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    r0, r1 = out[0], out[1]
    assert r0[:3] == (0, 2, 0) and r1[:3] == (1, 2, 1)
    # disjoint seeds, rank 0 is the single-GPU workload
    assert not set(r0[3]) & set(r1[3])
    from network_relaxation_gb300 import workloads

    assert r0[3] == [q["seed"] for q in workloads.c4_params(n=8)]
    # max over ranks of the step time, sum of the networks
    assert r0[4] == r1[4] == 20.0
    assert r0[5] == r1[5] == 16


def test_single_process_reduction_is_identity():
    from network_relaxation_gb300 import sharding

    assert sharding.reduce_timing(None, 3.5, 7) == (3.5, 7)
