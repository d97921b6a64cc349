"""Node reordering (nr_host_network_reorder, Morton and RCM) on the CPU.

Bonds and triples keep their order, so every node sums the same terms in
the same order: forces and energies of the reordered network equal the
original ones bit for bit, up to the permutation.
"""
import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle


def _shuffled_lattice(n, p, seed):
    h = nr.HostNetwork.lattice(n, n, p, 0.05, seed)
    a = h.arrays()
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(a["points"]))  # new -> old
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    hs = nr.HostNetwork.from_arrays(a["points"][perm], inv[a["edge_ij"]], a["edge_wrap"], a["offset"], a["edge_l0"])
    return hs.get_triples()


def _cross_fraction(a, parts=16):
    n = len(a["points"])
    b = -(-n // parts)
    ij = a["edge_ij"]
    return float(np.mean(ij[:, 0] // b != ij[:, 1] // b))


@pytest.mark.parametrize("method", ["morton", "rcm"])
def test_reorder_is_a_relabelling(method):
    h = _shuffled_lattice(48, 0.7, 3)
    a = h.arrays()
    h2 = nr.HostNetwork.from_arrays(a["points"], a["edge_ij"], a["edge_wrap"], a["offset"], a["edge_l0"]).get_triples()
    perm = h2.reorder(method)
    b = h2.arrays()
    assert sorted(perm.tolist()) == list(range(len(perm)))
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    assert np.array_equal(b["points"], a["points"][perm])
    assert np.array_equal(b["edge_ij"], inv[a["edge_ij"]])
    assert np.array_equal(b["edge_l0"], a["edge_l0"]) and np.array_equal(b["edge_wrap"], a["edge_wrap"])
    assert np.array_equal(b["tri_hjk"], inv[a["tri_hjk"]]) and np.array_equal(b["tri_wrap"], a["tri_wrap"])
    x = a["points"] + np.random.default_rng(1).normal(0, 0.03, a["points"].shape)
    fc = np.where(a["points"][:, 1] < a["miny"] + 1e-10, 0, 3).astype(np.uint8)
    F0 = oracle.Model(a, 1.0, 1e-2, fcodes=fc).forces(x)
    F1 = oracle.Model(b, 1.0, 1e-2, fcodes=fc[perm]).forces(x[perm])
    assert np.array_equal(F1, F0[perm])
    assert oracle.Model(a, 1.0, 1e-2, fcodes=fc).energies(x) == oracle.Model(b, 1.0, 1e-2, fcodes=fc[perm]).energies(x[perm])
    assert _cross_fraction(b) < 0.5 * _cross_fraction(a)


def test_reorder_mesh_composite():
    h = nr.HostNetwork.lattice_mesh(12, 9, 0.8, 0.1, 4)
    a = h.arrays()
    perm = h.reorder("morton")
    b = h.arrays()
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    assert np.array_equal(b["facets"], inv[a["facets"]]) and np.array_equal(b["mpairs"], inv[a["mpairs"]])
    gel_a, gel_b = oracle.mesh_gel(a, 0.5, 1.0, 0.02), oracle.mesh_gel(b, 0.5, 1.0, 0.02)
    x = a["points"] + np.random.default_rng(2).normal(0, 0.02, a["points"].shape) * 0
    F0 = oracle.Model(a, 1.0, 0.0, gel=gel_a).forces(x)
    F1 = oracle.Model(b, 1.0, 0.0, gel=gel_b).forces(x[perm])
    assert np.array_equal(F1, F0[perm])
