"""Linear response (sparse_relax.cpp) on the CPU: the oracle and the
library's host assembly against the reference.

Golden fixtures (tests/golden/spr/, made by the reference's own
sparse_relax.cpp with tests/golden/make_spr_golden.py) always; the
host-compiled reference live where its checkout exists.  Bars: stiffness
matrix entries (the library's and the oracle's), linearised energies and
the batch parser bit-exact; the protocol within the digits the reference's
energy (%12.10le) and .disp (%2.10le) files print.
"""
import json
import os

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "spr")
CASES = [(1.0, 0.0, 0.0), (1.0, 1e-2, 0.0), (0.5, 0.1, 0.05)]


def _net(name):
    ok, a = oracle.read_network(os.path.join(GOLD, name + ".dat"))
    assert ok
    return a


@pytest.mark.parametrize("name", ["s1", "s2"])
def test_stiffness_matches_golden(name):
    g = np.load(os.path.join(GOLD, "ref_spr.npz"))
    a = _net(name)
    h = nr.HostNetwork.read(os.path.join(GOLD, name + ".dat"))
    for c, (ks, kb, mu) in enumerate(CASES):
        ref = [g["%s_K%d_%s" % (name, c, k)] for k in ("rows", "cols", "vals")]
        for mine in (oracle.spr_stiffness(a, ks, kb, mu), nr.spr_assemble(h, ks, kb, mu)):
            assert all(np.array_equal(x, y) for x, y in zip(mine, ref)), (name, c)


@pytest.mark.parametrize("name", ["s1", "s2"])
def test_energies_match_golden(name):
    g = np.load(os.path.join(GOLD, "ref_spr.npz"))
    a = _net(name)
    assert oracle.spr_energies(a, 1.0, 1e-2, 0.05, g[name + "_u"]) == tuple(g[name + "_energies"])


@pytest.mark.parametrize("mode", ["affine", "top"])
def test_protocol_matches_golden(mode):
    d = os.path.join(GOLD, "ref_sweep_" + mode)
    prm = json.load(open(os.path.join(d, "params.json")))
    a = _net("s1")
    recs, fields = oracle.spr_protocol(a, prm["ks"], prm["kb"], prm["mu"], prm["compr"], prm["shear"],
                                       strain_mode=bool(prm["strain_mode"]), affine=bool(prm["affine"]))
    ref = np.loadtxt(os.path.join(d, "energies.txt"))
    mine = np.array([[r[0], r[1], r[3], r[4]] for r in recs])
    assert mine.shape == ref.shape
    assert np.allclose(mine[:, :2], ref[:, :2], rtol=0, atol=1e-8)
    assert np.allclose(mine[:, 2:], ref[:, 2:], rtol=2e-10, atol=1e-300)
    for k, f in enumerate(fields):
        u = np.loadtxt(os.path.join(d, "s1_%d.disp" % (k + 1))).reshape(-1)
        assert np.abs(u - f).max() <= 1e-10 * max(1.0, np.abs(f).max())
    resid = [float(ln.split(":")[1]) for ln in open(os.path.join(d, "log.txt"))]
    assert len(resid) == len(recs) and max(resid) < 1e-12


def test_spr_batch_parser_matches_golden():
    ref = json.load(open(os.path.join(GOLD, "ref_batch.json")))
    for name, r in ref.items():
        path = os.path.join(GOLD, "batch_files", name)
        try:
            s = nr.parse_spr_batch_file(path)
        except nr.NetRelaxError:
            assert not r["ok"], name
            continue
        assert r["ok"], name
        assert (s.base.decode(), s.tag.decode()) == (r["base"], r["tag"])
        assert [s.ks, s.kb, s.mu] == r["mech"] and list(s.compr) == r["compr"] and list(s.shear) == r["shear"]


@pytest.mark.parametrize("seed", range(12))
def test_live_reference_random_networks(seed, tmp_path):
    """Diluted lattices (with and without jitter) and Mikado networks (odd
    seeds: bonds of every direction, near-collinear segment pairs)."""
    if oracle.ref_spr_lib() is None and (oracle.build_ref() is None or oracle.ref_spr_lib() is None):
        pytest.skip("reference checkout not present")
    rng = np.random.default_rng(100 + seed)
    path = str(tmp_path / "r.dat")
    if seed % 2:
        h = nr.HostNetwork.mikado(int(rng.integers(60, 200)), 0.25, 1.0, 1e-3, seed + 1)
    else:
        h = nr.HostNetwork.lattice(int(rng.integers(5, 20)), int(rng.integers(4, 14)), float(rng.uniform(0.45, 1.0)),
                                   float(rng.choice([0.0, 0.05, 0.2])), seed + 1)
    h.write(path)
    r = oracle.RefSpr(path)
    a = _net_from(path)
    for ks, kb, mu in ((1.0, float(rng.uniform(0, 0.1)), float(rng.uniform(0, 0.2))),):
        ref = r.stiffness(ks, kb, mu)
        assert all(np.array_equal(x, y) for x, y in zip(oracle.spr_stiffness(a, ks, kb, mu), ref))
        assert all(np.array_equal(x, y) for x, y in zip(nr.spr_assemble(nr.HostNetwork.read(path), ks, kb, mu), ref))
        u = rng.normal(size=2 * len(a["points"]))
        assert oracle.spr_energies(a, ks, kb, mu, u) == r.energies(ks, kb, mu, u)


def _net_from(path):
    ok, a = oracle.read_network(path)
    assert ok
    return a


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_fire_energy_tends_to_the_linear_response(seed):
    """The two programs agree in the small-strain limit: the energy of the
    oracle's FIRE relaxation (large_strain_relax.cu) over the linear-response
    energy (sparse_relax.cpp) tends to 1, the difference shrinking in
    proportion to the strain (shear, then compression).  The lattices have
    unit rest lengths and straight rest triples: sparse_relax.cpp's spring
    constant is ks/l0 (SPR:292-303) where large_strain_relax.cu's is ks, so
    the two describe the same network only when l0 = 1."""
    h = nr.HostNetwork.lattice(12, 12, 0.8, 0.0, seed).get_triples()
    a = h.arrays()
    H = a["maxy"] - a["miny"]
    for shear in (True, False):
        dev = []
        for s, fcut in ((1e-4, 1e-13), (1e-5, 1e-14)):
            c_rng, s_rng = ([0.0, 0.0, 1.0], [s, s, 1.0]) if shear else ([s, s, 1.0], [0.0, 0.0, 1.0])
            recs, _ = oracle.spr_protocol(a, 1.0, 1e-2, 0.0, c_rng, s_rng, strain_mode=False)
            e_lin = recs[0][2]
            x0 = oracle.affine_displace(a["points"], a["miny"], H, s if shear else 0.0, 0.0 if shear else -s)
            _, _, _, rep = oracle.Model(a, 1.0, 1e-2).fire(x0, oracle.params(fcut=fcut, criterion="max",
                                                                            max_steps=400_000))
            assert rep.max_force < fcut
            dev.append((rep.e_stretch + rep.e_bend) / e_lin - 1)
        assert abs(dev[1]) < 2e-6, dev
        assert abs(dev[1]) < 0.2 * abs(dev[0]) + 1e-9, dev  # O(strain)
