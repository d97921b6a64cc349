"""Canonical arithmetic and known-answer tests of the oracle's physics (CPU).

The reference ships no tests; these known answers come from the model's
energy E = sum k/2 (|r|-l0)^2 + sum kb/2 (theta-theta0)^2.
"""
import math

import numpy as np
import pytest

import oracle


def ulps(a, b):
    return abs(a - b) / max(np.spacing(abs(b)), 5e-324)


def test_atan2_accuracy():
    rng = np.random.default_rng(0)
    pts = np.concatenate([rng.normal(size=(20000, 2)), rng.normal(size=(2000, 2)) * 1e-9,
                          np.stack([rng.normal(size=2000), rng.normal(size=2000) * 1e-12], 1)])
    worst = max(ulps(oracle.atan2(y, x), math.atan2(y, x)) for y, x in pts)
    assert worst <= 2.0
    assert oracle.atan2(0.0, 0.0) == 0.0
    assert oracle.atan2(1.0, 0.0) == math.atan2(1.0, 0.0)
    assert abs(oracle.atan2(0.0, -1.0) - math.pi) < 1e-15


def test_canonical_sum_structure():
    t = np.arange(1000, dtype=np.float64)
    assert oracle.canon_sum(t) == t.sum()
    rng = np.random.default_rng(1)
    x = rng.normal(size=70000)
    assert abs(oracle.canon_sum(x) - math.fsum(x)) < 1e-11
    assert oracle.canon_sum(np.zeros(0)) == 0.0
    # tile-padding: appending zeros does not change the bits
    assert oracle.canon_sum(x[:300]) == oracle.canon_sum(np.concatenate([x[:300], np.zeros(212)]))


def single_bond(delta, k=2.0):
    a = {"points": np.array([[0.0, 5.0], [1.0 + delta, 5.0]]), "edge_ij": np.array([[0, 1]], np.int32),
         "edge_l0": np.array([1.0]), "edge_wrap": np.zeros(1, np.int8), "tri_hjk": np.zeros((0, 3), np.int32),
         "tri_wrap": np.zeros((0, 2), np.int8), "offset": 100.0, "miny": 0.0, "maxy": 10.0}
    return oracle.Model(a, k, 0.0, np.array([3, 3], np.uint8)), a["points"]


def test_kat_single_bond_energy_and_force():
    m, x = single_bond(0.01)
    es, eb = m.energies(x)
    assert abs(es - 0.5 * 2.0 * 0.01**2) < 1e-17 and eb == 0.0
    F = m.forces(x)
    assert abs(F[0, 0] - 2.0 * 0.01) < 1e-15 and abs(F[1, 0] + 2.0 * 0.01) < 1e-15
    assert F[0, 1] == 0.0 and F[1, 1] == 0.0


def bent_triple(phi, kb=0.3):
    pts = np.array([[0.0, 5.0], [-1.0, 5.0], [math.cos(phi), 5.0 + math.sin(phi)]])
    a = {"points": pts, "edge_ij": np.zeros((0, 2), np.int32), "edge_l0": np.zeros(0), "edge_wrap": np.zeros(0, np.int8),
         "tri_hjk": np.array([[0, 1, 2]], np.int32), "tri_wrap": np.zeros((1, 2), np.int8), "offset": 100.0,
         "miny": 0.0, "maxy": 10.0}
    return oracle.Model(a, 0.0, kb, np.array([3, 3, 3], np.uint8)), pts


@pytest.mark.parametrize("phi", [1e-3, 0.2, -0.4])
def test_kat_bent_triple_energy(phi):
    m, x = bent_triple(phi)
    es, eb = m.energies(x)
    assert abs(eb - 0.5 * 0.3 * phi**2) <= 1e-14 * max(1.0, phi**2)


@pytest.mark.parametrize("model", ["bond", "triple", "lattice"])
def test_force_is_minus_gradient(model):
    if model == "bond":
        m, x = single_bond(0.03)
        x = x + np.array([[0.0, 0.02], [0.0, -0.01]])
    elif model == "triple":
        m, x = bent_triple(0.3)
        x = x + 0.01
    else:
        import network_relaxation_gb300 as nr

        a = nr.HostNetwork.lattice(6, 6, 0.8, 0.05, 3, line_triples=True).arrays()
        m = oracle.Model(a, 1.0, 0.1, np.full(36, 3, np.uint8))
        x = a["points"] + np.random.default_rng(2).normal(scale=0.05, size=a["points"].shape)
    F = m.forces(x)
    h = 1e-6
    for i in range(min(len(x), 12)):
        for c in range(2):
            xp, xm = x.copy(), x.copy()
            xp[i, c] += h
            xm[i, c] -= h
            g = (sum(m.energies(xp)) - sum(m.energies(xm))) / (2 * h)
            assert abs(F[i, c] + g) <= 1e-7 * max(1.0, abs(g)), (i, c, F[i, c], -g)


def test_homogeneous_lattice_affine_shear_is_equilibrium():
    """An undiluted lattice under affine simple shear is force-free inside
    (zero non-affinity): FIRE converges without moving any node."""
    import network_relaxation_gb300 as nr

    a = nr.HostNetwork.lattice(12, 12, 1.0, 0.0, 1).get_triples().arrays()
    H = a["maxy"] - a["miny"]
    m = oracle.Model(a, 1.0, 1e-2)
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.05 * H, 0.0)
    assert np.abs(m.forces(x0)).max() < 1e-13
    x, v, F, rep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max"))
    assert rep.converged and np.abs(x - x0).max() < 1e-12
    # elastic energy of affine simple shear of the triangular lattice:
    # sum over bonds k/2 (|r|-l0)^2 with exact image bond lengths
    p = a["points"]
    i, j = a["edge_ij"][:, 0], a["edge_ij"][:, 1]
    dx = x0[j, 0] + a["offset"] * a["edge_wrap"] - x0[i, 0]
    dy = x0[j, 1] - x0[i, 1]
    e_exact = 0.5 * np.sum((np.hypot(dx, dy) - a["edge_l0"]) ** 2)
    assert abs(rep.e_stretch - e_exact) <= 1e-12 * e_exact
    assert rep.e_bend < 1e-3 * rep.e_stretch


def test_clamped_rows_never_move():
    import network_relaxation_gb300 as nr

    a = nr.HostNetwork.lattice(10, 10, 0.7, 0.0, 4).get_triples().arrays()
    H = a["maxy"] - a["miny"]
    m = oracle.Model(a, 1.0, 1e-3)
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.05 * H, 0.0)
    x, v, F, rep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max"))
    clamped = m.fcodes == 0
    assert clamped.sum() == 20
    assert np.array_equal(x[clamped], x0[clamped])
    assert np.all(F[clamped] == 0)
