"""Synthetic network generators (no reference counterpart: the reference
ships no inputs).  Invariants of the Mikado generator (config C3) checked
on the host with the oracle's force."""
import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle


@pytest.fixture(scope="module")
def small():
    h = nr.HostNetwork.mikado(600, 0.1, 1.0, 1e-3, 3)
    return h, h.arrays()


def test_mikado_topology(built, small):
    _, a = small
    n = len(a["points"])
    assert n > 500 and len(a["edge_l0"]) > n and len(a["tri_hjk"]) > 0
    assert a["miny"] == 0.0 and a["maxy"] == 1.0 and a["offset"] == 1.0
    x, y = a["points"][:, 0], a["points"][:, 1]
    assert x.min() >= 0.0 and x.max() < 1.0 and y.min() >= 0.0 and y.max() <= 1.0
    assert np.all(np.diff(y) >= 0)  # numbered by y: node blocks are horizontal bands
    deg = np.bincount(a["edge_ij"].ravel(), minlength=n)
    clamped = (y == 0.0) | (y == 1.0)
    assert deg[~clamped].min() >= 2  # dangling ends pruned
    assert np.all(deg[clamped] == 1)  # fibers cut at y = 0 / 1 end there


def test_mikado_geometry_and_stiffness(built, small):
    _, a = small
    P, ij, w = a["points"], a["edge_ij"], a["edge_wrap"]
    r = P[ij[:, 1]] - P[ij[:, 0]]
    r[:, 0] += w * a["offset"]
    L = np.hypot(r[:, 0], r[:, 1])
    assert L.max() <= 0.1 + 1e-12 and np.abs(L - a["edge_l0"]).max() < 1e-15
    np.testing.assert_allclose(a["bond_k"] * a["edge_l0"], 1.0, rtol=1e-15)
    # triples: consecutive segments of one fiber, straight at rest
    h, j, k = a["tri_hjk"].T
    assert np.abs(a["tri_phi0"]).max() < 1e-9
    m = oracle.Model(a, 1.0, 1.0)
    F = m.forces(P)
    assert np.abs(F).max() < 1e-9  # rest state force-free (k up to 1/l0_min)
    es, eb = m.energies(P)
    assert es < 1e-25 and eb < 1e-25


def test_mikado_seeded(built):
    a1 = nr.HostNetwork.mikado(300, 0.1, 1.0, 1e-3, 11).arrays()
    a2 = nr.HostNetwork.mikado(300, 0.1, 1.0, 1e-3, 11).arrays()
    a3 = nr.HostNetwork.mikado(300, 0.1, 1.0, 1e-3, 12).arrays()
    assert np.array_equal(a1["points"], a2["points"]) and np.array_equal(a1["edge_ij"], a2["edge_ij"])
    assert len(a1["points"]) != len(a3["points"]) or not np.array_equal(a1["points"], a3["points"])


def test_mikado_c3_size(built):
    """C3: unit box, fibre length 0.05, 15 850 fibres -> ~2e5 nodes."""
    i = nr.HostNetwork.mikado(15850, 0.05, 1.0, 1e-5, 3).info()
    assert 1.8e5 < i.n_points < 2.2e5 and 3.4e5 < i.n_edges < 4.2e5 and 3.3e5 < i.n_triples < 4.1e5


def test_mikado_bad_arguments(built):
    with pytest.raises(nr.NetRelaxError):
        nr.HostNetwork.mikado(0, 0.1, 1.0, 1e-3, 1)
    with pytest.raises(nr.NetRelaxError):
        nr.HostNetwork.mikado(100, 0.7, 1.0, 1e-3, 1)
