"""The tuning table steers the launches the library makes (GB300).

The library reads every launch-policy knob through the table it loads for
the device (tuning/<device name>.txt beside libnetrelax.so, written by the
autotuner).  These tests check that the committed table is the one loaded
on this device, that a table's entries change the plan that the library
reports AND runs, and that every plan gives the oracle's bits (FP64).
"""
import os
import re

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE_DIR = os.path.join(ROOT, "network_relaxation_gb300", "tuning")
KNOBS = ("NR_FP64_CLUSTER_NODES", "NR_FP64_CLUSTER", "NR_FP64_KERNEL", "NR_FP64_BATCH_CLUSTER", "NR_CLUSTER",
         "NR_TUNING_FILE")
FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)


@pytest.fixture
def lib(cuda, monkeypatch):
    """The library with no knob in the environment; the table in effect
    before the test is loaded again after it."""
    for k in KNOBS:
        monkeypatch.delenv(k, raising=False)
    L = nr.lib()
    before = L.nr_tuning_source().decode()
    yield L
    if before:
        assert L.nr_tuning_load(before.encode()) >= 0


def device_table():
    import torch

    name = re.sub(r"[^a-z0-9]", "_", torch.cuda.get_device_name(0).lower())
    return os.path.join(TABLE_DIR, name + ".txt")


def test_committed_table_is_loaded_for_this_device(lib):
    path = device_table()
    if not os.path.exists(path):
        pytest.skip("no table committed for " + os.path.basename(path))
    assert os.path.realpath(lib.nr_tuning_source().decode()) == os.path.realpath(path)
    # every entry of the file is what the library reads
    for line in open(path):
        line = line.split("#")[0].split()
        if line:
            v = lib.nr_tuning_value(line[0].encode())
            assert (v != v) if line[1].isalpha() else v == float(line[1]), line


def relax_c1(net, a):
    H = a["maxy"] - a["miny"]
    net.affine_displace(a["miny"], H, 0.01 * H, 0.0)
    return net.relax(nr.fire_params(fcut=1e-10, criterion="max", **FIRE))


def test_table_entries_change_the_plan_and_keep_the_bits(lib, tmp_path):
    h = nr.HostNetwork.lattice(32, 32, 0.65, 0.0, 1)
    h.get_triples()
    a = h.arrays()
    H = a["maxy"] - a["miny"]
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.01 * H, 0.0)
    xo, _, _, orep = oracle.Model(a, 1.0, 1e-3).fire(x0, oracle.params(fcut=1e-10, criterion="max", **FIRE))
    tables = {
        "grid": ("NR_FP64_CLUSTER_NODES 0\n", "k_fire_grid"),
        "dsm4": ("NR_FP64_CLUSTER_NODES 4096\nNR_FP64_CLUSTER 4\nNR_FP64_KERNEL dsm\n", "k_fire_dsm64 cluster=4"),
        "l2_8": ("NR_FP64_CLUSTER_NODES 4096\nNR_FP64_CLUSTER 8\nNR_FP64_KERNEL l2\n", "k_fire_cluster cluster=8"),
    }
    for name, (text, want) in tables.items():
        t = tmp_path / (name + ".txt")
        t.write_text(text)
        assert lib.nr_tuning_load(str(t).encode()) > 0
        net = nr.Network(h, ks=1.0, kb=1e-3)
        assert net.plan("fp64").startswith(want), (name, net.plan("fp64"))
        rep = relax_c1(net, a)
        assert rep.status == nr.NR_OK and rep.steps == orep.steps, name
        assert np.array_equal(net.positions(), xo), name
        net.close()


def test_table_sets_the_batch_cluster(lib, tmp_path):
    hs = []
    for s in range(3):
        h = nr.HostNetwork.lattice(24, 24, 0.7, 0.0, 10 + s)
        h.get_triples()
        hs.append(h)
    for c in (2, 8):
        t = tmp_path / "b.txt"
        t.write_text("NR_CLUSTER %d\nNR_FP64_BATCH_CLUSTER %d\n" % (c, c))
        assert lib.nr_tuning_load(str(t).encode()) == 2
        b = nr.Batch(hs, ks=1.0, kb=1e-3)
        assert ("cluster=%d" % c) in b.plan("mixed"), b.plan("mixed")
        assert ("cluster=%d" % c) in b.plan("fp64"), b.plan("fp64")


def test_table_sets_the_single_cta_launch(lib, tmp_path):
    """NR_SOLO_CTAS sizes the one-network-per-CTA launch beside the
    clusters (default: the SMs the clusters leave)."""
    hs = []
    for L in (60, 60, 20, 20, 20):  # two networks on clusters, three small ones on single CTAs
        h = nr.HostNetwork.lattice(L, L, 0.7, 0.0, 30 + L)
        h.get_triples()
        hs.append(h)
    b = nr.Batch(hs, ks=1.0, kb=1e-3)
    plan = b.plan("mixed")
    if "solo_networks=0" in plan:
        pytest.skip("no single-CTA split for this batch: " + plan)
    t = tmp_path / "s.txt"
    t.write_text("NR_SOLO_CTAS 7\n")
    assert lib.nr_tuning_load(str(t).encode()) == 1
    assert "solo_ctas=7" in b.plan("mixed"), b.plan("mixed")
