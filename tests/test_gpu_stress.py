"""Stress outputs on the GPU against the oracle's restatement (or_virial):
sigma = W / A with the canonical sums, so the FP64 path's stress is
bit-identical to the oracle's at the same positions -- after an FP64
relaxation (grid kernel), after a batch relaxation (FP64 batch kernel and
mixed precision, computed from each network's returned positions), from
nr_stress, and in the records of the strain sweep."""
import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)


def _oracle_stress(a, ks, kb, x):
    A = a["offset"] * (a["maxy"] - a["miny"])
    return oracle.Model(a, ks, kb).virial(x) * (1.0 / A)


def test_fp64_relax_stress_bitexact(cuda):
    h = nr.HostNetwork.lattice(24, 24, 0.7, 0.05, 31, line_triples=True)
    a = h.arrays()
    net = nr.Network(h, 1.0, 1e-3)
    H = net.maxy - net.miny
    net.affine_displace(net.miny, H, 0.03 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="fp64", **FIRE))
    assert rep.status == nr.NR_OK
    x = net.positions()
    s = _oracle_stress(a, 1.0, 1e-3, x)
    assert (rep.stress_xx, rep.stress_yy, rep.stress_xy) == tuple(s)
    assert rep.stress_xy > 0
    st, (es, eb) = net.stress()
    assert tuple(st) == tuple(s) and (es, eb) == (rep.e_stretch, rep.e_bend)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_stress_matches_oracle_at_returned_positions(cuda, precision):
    rng = np.random.default_rng(9)
    hosts, arrs, kb = [], [], []
    for i, L in enumerate([18, 30, 12]):
        hh = nr.HostNetwork.lattice(L, L, 0.72, 0.0, 40 + i).get_triples()
        hosts.append(hh)
        arrs.append(hh.arrays())
        kb.append(float(10 ** rng.uniform(-3, -2)))
    kb = np.array(kb)
    b = nr.Batch(hosts, 1.0, kb)
    b.affine_displace(0.02 * (b.maxy - b.miny), 0.0)
    reps = b.relax(nr.fire_params(fcut=1e-10, criterion="max", precision=precision, **FIRE))
    X = b.positions()
    for i, a in enumerate(arrs):
        assert reps[i].status == nr.NR_OK
        x = X[b.offsets[i]:b.offsets[i + 1]]
        s = _oracle_stress(a, 1.0, kb[i], x)
        assert (reps[i].stress_xx, reps[i].stress_yy, reps[i].stress_xy) == tuple(s)


def test_sweep_records_carry_stress(cuda):
    h = nr.HostNetwork.lattice(16, 16, 0.75, 0.0, 5).get_triples()
    a = h.arrays()
    net = nr.Network(h, 1.0, 1e-3)
    prm = nr.fire_params(fcut=1e-10, criterion="max", precision="fp64", **FIRE)
    recs, pos = net.sweep((0.0, 0.0, 0.0), (0.01, 0.03, 0.01), prm, keep_positions=True)
    assert len(recs) == 3
    for r, x in zip(recs, pos):
        s = _oracle_stress(a, 1.0, 1e-3, x)
        assert (r.stress_xx, r.stress_yy, r.stress_xy) == tuple(s)
    # the shear stress grows with the strain
    assert recs[0].stress_xy < recs[1].stress_xy < recs[2].stress_xy


def test_lsrelax_stress_columns(cuda, tmp_path):
    """lsrelax --stress appends sigma_xy and sigma_yy to every _edata line;
    without it the file keeps the reference's five columns, and the first
    five columns are the same bytes either way."""
    import os
    import shutil
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = os.path.join(root, "network_relaxation_gb300", "lsrelax")
    shutil.copy(os.path.join(root, "tests", "golden", "small.dat"), tmp_path / "net.dat")
    (tmp_path / "batch.txt").write_text("%s t\n1.0 0.001\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-10 1000000\n"
                                        "0 0 0\n0.01 0.03 0.01\n" % (tmp_path / "net"))
    env = dict(os.environ)
    runs = {}
    for flag in ([], ["--stress"]):
        r = subprocess.run([exe, "-b", str(tmp_path / "batch.txt")] + flag, capture_output=True, text=True, env=env)
        assert r.returncode == 0, r.stderr
        runs[bool(flag)] = (tmp_path / "net_t_edata.txt").read_text().splitlines()
    plain, withs = runs[False], runs[True]
    assert len(plain) == len(withs) == 3
    for a, b in zip(plain, withs):
        assert len(a.split("\t")) == 5 and len(b.split("\t")) == 7
        assert b.startswith(a + "\t")
    # the stress columns are the sweep's records, printed
    h = nr.HostNetwork.read(str(tmp_path / "net.dat")).get_triples()
    net = nr.Network(h, 1.0, 1e-3)
    prm = nr.fire_params(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10,
                         max_steps=1000000, criterion="rms", precision="fp64")
    recs, _ = net.sweep((0.0, 0.0, 0.0), (0.01, 0.03, 0.01), prm)
    for line, r in zip(withs, recs):
        cols = line.split("\t")
        assert cols[5] == "%12.10e" % r.stress_xy and cols[6] == "%12.10e" % r.stress_yy
