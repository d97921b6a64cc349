"""Pins the oracle to the reference.

Against the golden fixtures (always; produced by the reference's own
large_strain_relax.cu compiled for the host, tests/golden/make_golden.py) and,
where the reference checkout exists, against that compiled reference live.
Bars: topology, affine start and reader behaviour bit-exact; relaxed energy
within 1e-10 relative, positions within 1e-8 lattice spacings.
"""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIRE = [0.1, 0.99, 0.1, 1.1, 0.5]


def _gold_c1():
    return np.load(os.path.join(GOLD, "ref_c1.npz"))


def test_reader_and_triples_match_golden():
    g = _gold_c1()
    ok, a = oracle.read_network(os.path.join(GOLD, "c1.dat"))
    assert ok
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a[k], g[k]), k
    assert a["offset"] == g["offset"] and a["miny"] == g["miny"] and a["maxy"] == g["maxy"]
    fc = np.where((a["points"][:, 1] < a["miny"] + 1e-10) | (a["points"][:, 1] > a["maxy"] - 1e-10), 0, 3)
    assert np.array_equal(fc, g["fcodes"])


def test_reader_edge_cases_match_golden():
    ref = json.load(open(os.path.join(GOLD, "ref_readers.json")))
    for name, r in ref.items():
        ok, a = oracle.read_network(os.path.join(GOLD, "edge_cases", name))
        assert ok == r["ok"], name
        assert len(a["points"]) == r["n_points"] and len(a["edge_l0"]) == r["n_edges"], name
        assert len(a["tri_hjk"]) == r["n_triples"], name
        assert a["points"].tolist() == r["points"], name
        assert a["edge_ij"].tolist() == r["edge_ij"] and a["edge_wrap"].tolist() == r["edge_wrap"], name
        assert [float(v).hex() for v in a["edge_l0"]] == r["edge_l0"], name
        assert a["tri_hjk"].tolist() == r["tri_hjk"] and a["tri_wrap"].tolist() == r["tri_wrap"], name
        if r["n_points"]:
            assert float(a["miny"]).hex() == r["miny"] and float(a["maxy"]).hex() == r["maxy"], name


def test_affine_start_matches_golden():
    g = _gold_c1()
    H = float(g["maxy"] - g["miny"])
    x0 = oracle.affine_displace(g["points"], float(g["miny"]), H, 0.01 * H, 0.0)
    assert np.array_equal(x0, g["x_affine"])


def test_fire_matches_golden_reference_run():
    """run_fire_md of the reference vs the oracle on config C1's first shear
    step (32x32, p=0.65, kappa=1e-3, RMS criterion)."""
    g = _gold_c1()
    a = {k: g[k] for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap")}
    a.update(offset=float(g["offset"]), miny=float(g["miny"]), maxy=float(g["maxy"]))
    m = oracle.Model(a, 1.0, 1e-3, g["fcodes"])
    x, v, F, rep = m.fire(g["x_affine"], oracle.params(fcut=float(g["fcut"]), criterion="rms"))
    r = g["report"]
    assert abs(rep.e_stretch - r[1]) <= 1e-10 * abs(r[1])
    assert abs(rep.e_bend - r[2]) <= 1e-10 * abs(r[2])
    assert np.abs(x - g["x_relaxed"]).max() <= 1e-8  # unit lattice spacing
    assert rep.rms_force <= float(g["fcut"])
    assert abs(rep.steps - int(g["steps"])) <= max(5, int(0.01 * int(g["steps"])))


def test_sweep_matches_golden_reference_outputs():
    """do_relaxation_run's edata / pos outputs for small.dat vs the oracle's
    protocol restatement (energies 1e-10 relative, positions 1e-8)."""
    ok, a = oracle.read_network(os.path.join(GOLD, "small.dat"))
    assert ok
    H = a["maxy"] - a["miny"]
    m = oracle.Model(a, 1.0, 1e-3)
    recs, pos, _ = m.sweep(a["points"], a["miny"], H, oracle.params(fcut=1e-12, criterion="rms"),
                           [0.01, 0.02, 0.01], [0.01, 0.03, 0.01])
    edata = np.loadtxt(os.path.join(GOLD, "ref_sweep", "small_edata.txt"))
    assert len(recs) == len(edata) == 5
    for r, e in zip(recs, edata):
        assert abs(r[0] - e[0]) < 1e-9 and abs(r[1] - e[1]) < 1e-9
        # edata is printed with 9-11 significant digits
        assert abs(r[2] - e[2]) <= 1e-8 * abs(e[2]) + 1e-18
        assert abs(r[3] - e[3]) <= 1e-8 * abs(e[3]) + 1e-18
    shear = [i for i, r in enumerate(recs) if r[7] == 1]
    for k, i in enumerate(shear):
        ref_pos = np.loadtxt(os.path.join(GOLD, "ref_sweep", "small_%d.pos" % (k + 1)))
        assert np.abs(pos[i] - ref_pos).max() <= 1e-8
    log = open(os.path.join(GOLD, "ref_sweep", "small_log.txt")).read().splitlines()
    assert len(log) == 5 and all(line.startswith("Convergence reached") for line in log)
    steps = [int(line.split("Steps: ")[1].split(",")[0]) for line in log]
    for r, s in zip(recs, steps):
        assert abs(int(r[6]) - s) <= max(5, s // 100)


@pytest.fixture(scope="module")
def ref():
    if oracle.build_ref() is None or oracle.ref_lib() is None:
        pytest.skip("reference checkout not available (golden fixtures cover this case)")
    return oracle.ref_lib()


@pytest.mark.parametrize("n,p,seed", [(10, 0.9, 1), (24, 0.65, 2), (33, 0.55, 3), (16, 1.0, 4)])
def test_live_reference_topology_bitexact(ref, tmp_path, n, p, seed):
    import network_relaxation_gb300 as nr

    path = str(tmp_path / "net.dat")
    nr.HostNetwork.lattice(n, n, p, 0.0, seed).write(path)
    ok, a = oracle.read_network(path)
    rok, r = oracle.ref_read_network(path)
    assert ok and rok
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a[k], r[k]), k


@pytest.mark.parametrize("n,p,seed,kb,gamma", [(16, 0.7, 5, 1e-3, 0.02), (20, 0.62, 6, 1e-2, 0.05), (12, 0.8, 7, 0.0, 0.01)])
def test_live_reference_fire(ref, tmp_path, n, p, seed, kb, gamma):
    import network_relaxation_gb300 as nr

    path = str(tmp_path / "net.dat")
    nr.HostNetwork.lattice(n, n, p, 0.0, seed).write(path)
    rok, r = oracle.ref_read_network(path, want_triples=kb > 0)
    N = len(r["points"])
    H = r["maxy"] - r["miny"]
    fc = np.where((r["points"][:, 1] < r["miny"] + 1e-10) | (r["points"][:, 1] > r["maxy"] - 1e-10), 0, 3).astype(np.uint8)
    x0 = oracle.ref_affine_displace(r["points"], r["miny"], H, gamma * H, 0.0)
    assert np.array_equal(x0, oracle.affine_displace(r["points"], r["miny"], H, gamma * H, 0.0))
    fcut = 1e-10 / np.sqrt(2 * N)
    xr, rep, steps = oracle.ref_run_fire_md(r, x0, 1.0, kb, fc, FIRE, 1.0, fcut, 10**6, 5)
    x, v, F, orep = oracle.Model(r, 1.0, kb, fc).fire(x0, oracle.params(fcut=fcut, criterion="rms"))
    assert abs(orep.e_stretch - rep[1]) <= 1e-10 * abs(rep[1]) + 1e-20
    assert abs(orep.e_bend - rep[2]) <= 1e-10 * abs(rep[2]) + 1e-20
    assert np.abs(x - xr).max() <= 1e-8
