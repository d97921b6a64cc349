"""Gel coupling (network_mesh_relax.cu) on the GPU vs the oracle.

The FP64 path keeps the oracle's arithmetic for the gel terms too (the
reference's own expression order, no fused operations, element terms added
per node in element order, duplicate vertices summed), so forces, inverse
matrices, dilation, trajectories, step counts and all three energies agree
BIT-FOR-BIT with the oracle; against the reference's golden runs the bars of
tests/test_mesh.py apply.
"""
import json
import math
import os
import shutil

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "mesh")
FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)
FIRE_LIST = [0.1, 0.99, 0.1, 1.1, 0.5]


def composite(nx, ny, p, jitter, seed, kb):
    h = nr.HostNetwork.lattice_mesh(nx, ny, p, jitter, seed)
    if kb > 0:
        h.get_triples()
    return h, h.arrays()


def perturbed(a, seed, scale=0.04, tie_pairs=True):
    rng = np.random.default_rng(seed)
    fc = nr_fcodes(a)
    x = a["points"] + rng.normal(0.0, scale, a["points"].shape) * (fc[:, None] > 0)
    if tie_pairs:
        for i, j in a["mpairs"]:
            x[j] = x[i] + [a["offset"], 0.0]
    return x


def nr_fcodes(a):
    y = a["points"][:, 1]
    return np.where((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10), 0, 3).astype(np.uint8)


@pytest.mark.parametrize("ks,kb,tie", [(0.0, 0.0, True), (1.0, 0.0, True), (1.0, 1e-2, True), (1.0, 1e-2, False)])
def test_mesh_forces_and_energies_bitwise(cuda, ks, kb, tie):
    h, a = composite(16, 12, 0.75, 0.1, 3, kb)
    gel = oracle.mesh_gel(a, 0.6, 1.5, 0.08)
    net = nr.Network(h, ks=ks, kb=kb)
    net.set_gel(0.6, 1.5, 0.08)
    x = perturbed(a, 7, tie_pairs=tie)
    net.set_positions(x)
    m = oracle.Model(a, ks, kb, gel=gel)
    F, Fo = net.forces(), m.forces(x)
    assert np.array_equal(F, Fo), np.abs(F - Fo).max()
    es, eb, eg = net.mesh_energies()
    eso, ebo = m.energies(x)
    assert (es, eb, eg) == (eso, ebo, m.gel_energy(x))


def test_inv_mats_dropin_and_dilate_bitwise(cuda):
    import torch

    ok, a = oracle.read_network_mesh(os.path.join(GOLD, "m1.nmc"))
    g = np.load(os.path.join(GOLD, "ref_m1.npz"))
    d_pos = torch.tensor(a["points"].reshape(-1), dtype=torch.float64, device=cuda)
    d_fac = torch.tensor(a["facets"].reshape(-1), dtype=torch.int32, device=cuda)
    d_inv = torch.zeros(6 * len(a["facets"]), dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()
    nr.get_inv_mats(len(a["facets"]), d_pos.data_ptr(), d_fac.data_ptr(), d_inv.data_ptr())
    torch.cuda.synchronize()
    inv = d_inv.cpu().numpy().reshape(-1, 6)
    assert np.array_equal(inv, oracle.inv_mats(a["points"], a["facets"]))
    assert np.array_equal(inv, g["inv_mats"])  # the reference's get_inv_mats, host-compiled
    h = nr.HostNetwork.read_mesh(os.path.join(GOLD, "m1.nmc"))
    net = nr.Network(h, ks=1.0, kb=0.0)
    net.dilate(a["minx"], a["miny"], math.sqrt(1.07))
    assert np.array_equal(net.positions(), oracle.dilate(a["points"], a["minx"], a["miny"], math.sqrt(1.07)))


@pytest.mark.parametrize("ks,kb,seed", [(1.0, 1e-3, 1), (1.0, 0.0, 2), (0.0, 0.0, 3)])
def test_mesh_relax_bitwise(cuda, ks, kb, seed):
    h, a = composite(20, 14, 0.7, 0.12, seed, kb)
    gel = oracle.mesh_gel(a, 0.4, 1.0, 0.03)
    net = nr.Network(h, ks=ks, kb=kb)
    net.set_gel(0.4, 1.0, 0.03)
    H = a["maxy"] - a["miny"]
    net.affine_displace(a["miny"], H, 0.03 * H, -0.01 * H)
    N = len(a["points"])
    fcut = 1e-10
    rep = net.relax(nr.fire_params(fcut=fcut, criterion="rms", max_steps=200000, **FIRE))
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.03 * H, -0.01 * H)
    xo, vo, Fo, orep = oracle.Model(a, ks, kb, gel=gel).fire(
        x0, oracle.params(fcut=fcut, criterion="rms", max_steps=200000, **FIRE))
    assert rep.status == nr.NR_OK and orep.converged
    assert rep.steps == orep.steps
    assert np.array_equal(net.positions(), xo)
    assert (rep.e_stretch, rep.e_bend, rep.e_gel) == (orep.e_stretch, orep.e_bend, orep.e_gel)
    assert rep.rms_force == orep.rms_force and N > 0


def test_mesh_relax_matches_golden_reference_run(cuda):
    h = nr.HostNetwork.read_mesh(os.path.join(GOLD, "m1.nmc")).get_triples()
    g = np.load(os.path.join(GOLD, "ref_m1.npz"))
    net = nr.Network(h, ks=1.0, kb=1e-2)
    net.set_gel(0.7, 2.0, 0.05)
    net.set_positions(g["x_affine"])
    rep = net.relax(nr.fire_params(fcut=1e-9, criterion="rms", max_steps=200000, **FIRE))
    r = g["fire_report"]
    assert rep.steps == int(g["fire_steps"])
    total = sum(r[1:])
    for mine, theirs in zip((rep.e_stretch, rep.e_bend, rep.e_gel), r[1:]):
        assert abs(mine - theirs) <= 1e-12 * total
    assert np.abs(net.positions() - g["fire_pos"]).max() < 1e-10


def _prepared(path, prm):
    s = math.sqrt(1 + prm["dilation"])
    h = nr.HostNetwork.read_mesh(path)
    i, m = h.info(), h.mesh_info()
    h.set_offset(i.offset * s)
    if prm["kb"] > 0:
        h.get_triples()
    net = nr.Network(h, ks=prm["ks"], kb=prm["kb"])
    area = (m.maxx - m.minx) * (i.maxy - i.miny)
    pref = net.mesh_prepare(prm["smod"], prm["bmod"], prm["dilation"], area)
    return net, pref, (i.maxy - i.miny) * s, i.miny


def test_mesh_protocol_bitwise_and_golden(cuda):
    """do_relaxation_run's set-up and loops through the library API vs the
    oracle (bitwise) and vs the reference's edata / .pos files."""
    from test_mesh import _oracle_protocol

    d = os.path.join(GOLD, "ref_sweep")
    prm = json.load(open(os.path.join(d, "params.json")))
    path = os.path.join(GOLD, "sweep.nmc")
    net, pref, height, miny = _prepared(path, prm)
    recs_o, shp_o, pref_o = _oracle_protocol(path, prm)
    assert pref == pref_o
    fp = nr.fire_params(*prm["fire"], nmin=prm["nmin"], mass=prm["mass"], fcut=prm["fcut"], max_steps=prm["nmax"],
                        criterion="rms")
    recs, pos = net.mesh_sweep(prm["compr"], prm["shear"], height, fp, miny=miny, keep_positions=True)
    assert len(recs) == len(recs_o)
    for r, o in zip(recs, recs_o):
        assert (r.curr_disp, r.max_comp, r.e_stretch, r.e_bend, r.e_gel, r.rms_force, r.steps) == \
            (o[0], o[1], o[2], o[3], o[4], o[5], int(o[7]))
    for k, r in enumerate(recs):
        if r.is_shear:
            assert np.array_equal(pos[k], shp_o[k])
    ref = np.loadtxt(os.path.join(d, "sweep_edata.txt"))
    mine = np.array([[r.curr_disp, r.max_comp, r.e_stretch, r.e_bend, r.e_gel, r.e_stretch + r.e_bend + r.e_gel]
                     for r in recs])
    assert np.allclose(mine, ref, rtol=2e-8, atol=1e-8)


def test_nmrelax_cli_matches_golden(cuda, tmp_path):
    d = os.path.join(GOLD, "ref_sweep")
    prm = json.load(open(os.path.join(d, "params.json")))
    shutil.copy(os.path.join(GOLD, "sweep.nmc"), tmp_path / "sweep.nmc")
    batch = tmp_path / "batch.txt"
    batch.write_text("%s\n%r %r %r %r %r\n%s\n%d %r %r %d\n%r %r %r\n%r %r %r\n" % (
        tmp_path / "sweep", prm["ks"], prm["kb"], prm["bmod"], prm["smod"], prm["dilation"],
        " ".join(repr(v) for v in prm["fire"]), prm["nmin"], prm["mass"], prm["fcut"], prm["nmax"],
        *prm["compr"], *prm["shear"]))
    assert nr.nmrelax_main(["-b", str(batch)]) == 0
    mine = np.loadtxt(tmp_path / "sweep_edata.txt")
    ref = np.loadtxt(os.path.join(d, "sweep_edata.txt"))
    assert mine.shape == ref.shape and np.allclose(mine, ref, rtol=2e-8, atol=1e-8)
    log = [ln for ln in open(tmp_path / "sweep_log.txt") if not ln.startswith("Elapsed")]
    ref_log = open(os.path.join(d, "sweep_log.txt")).readlines()
    assert [ln.split(",")[0] for ln in log] == [ln.split(",")[0] for ln in ref_log]  # verdict and step count
    for k in (1, 2, 3):
        P = np.loadtxt(tmp_path / ("sweep_%d.pos" % k))
        assert np.abs(P - np.loadtxt(os.path.join(d, "sweep_%d.pos" % k))).max() < 1e-8


def test_mesh_run_fire_md_dropin(cuda):
    """network_mesh_relax.cu's run_fire_md argument list on torch arrays."""
    import torch

    h, a = composite(14, 10, 0.8, 0.1, 12, 1e-3)
    N = len(a["points"])
    H = a["maxy"] - a["miny"]
    fc = nr_fcodes(a)
    inv = oracle.inv_mats(a["points"], a["facets"])
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.02 * H, 0.0)
    t = lambda v, dt: torch.tensor(np.ascontiguousarray(v).reshape(-1), dtype=dt, device=cuda)  # noqa: E731
    d_pos = t(x0, torch.float64)
    d_vel, d_f = torch.zeros_like(d_pos), torch.zeros_like(d_pos)
    arrays = [t(a["edge_ij"], torch.int32), t(a["edge_l0"], torch.float64), t(a["edge_wrap"], torch.int8),
              t(a["tri_hjk"], torch.int32), t(a["tri_wrap"], torch.int8), t(a["facets"], torch.int32),
              t(a["areas"], torch.float64), t(inv, torch.float64), t(a["mpairs"], torch.int32)]
    d_fc = t(fc, torch.uint8)
    torch.cuda.synchronize()
    ptr = [v.data_ptr() for v in arrays]
    st, report, steps = nr.mesh_run_fire_md(
        2 * N, len(a["edge_l0"]), len(a["tri_hjk"]), len(a["facets"]), a["offset"], 1.0, 1e-3, 0.5, 1.2, 0.02,
        d_pos.data_ptr(), d_vel.data_ptr(), d_f.data_ptr(), *ptr[:8], ptr[8], len(a["mpairs"]), d_fc.data_ptr(),
        FIRE_LIST, 1.0, 1e-9, 10**6, 5)
    gel = oracle.mesh_gel(a, 0.5, 1.2, 0.02, inv=inv)
    xo, vo, Fo, orep = oracle.Model(a, 1.0, 1e-3, fc, gel=gel).fire(x0, oracle.params(fcut=1e-9, criterion="rms",
                                                                                      **FIRE))
    assert st == nr.NR_OK and steps == orep.steps
    assert np.array_equal(d_pos.cpu().numpy().reshape(-1, 2), xo)
    assert np.array_equal(d_f.cpu().numpy().reshape(-1, 2), Fo)
    assert report == [orep.rms_force, orep.e_stretch, orep.e_bend, orep.e_gel]


def test_mesh_rejections(cuda):
    h, a = composite(8, 6, 0.8, 0.0, 2, 0.0)
    net = nr.Network(h, ks=1.0, kb=0.0)
    net.set_gel(0.5, 1.0, 0.0)
    with pytest.raises(nr.NetRelaxError) as e:
        net.relax(nr.fire_params(precision="mixed"))
    assert e.value.status == nr.NR_ERR_INVALID
    bad = nr.HostNetwork.lattice_mesh(8, 6, 0.8, 0.0, 2)
    bad.set_mesh(a["facets"], a["areas"], [[0, 1], [1, 2]])  # vertex 1 in two pairs
    net2 = nr.Network(bad, ks=1.0, kb=0.0)
    with pytest.raises(nr.NetRelaxError) as e:
        net2.set_gel(0.5, 1.0, 0.0)
    assert e.value.status == nr.NR_ERR_INVALID
    net2.set_gel(0.5, 0.0, 0.0)  # bmod = 0: no gel, accepted (network_mesh_relax.cu:908)


def test_mesh_large_properties(cuda):
    """A 200 x 150 composite (30k nodes, 60k triangles) through one shear
    step on the grid kernel: converged, duplicate vertices stay exactly one
    period apart in y and receive identical forces, the gel carries energy."""
    h, a = composite(200, 150, 0.7, 0.1, 4, 0.0)
    net = nr.Network(h, ks=1.0, kb=0.0)
    net.set_gel(0.3, 1.0, 0.02)
    H = a["maxy"] - a["miny"]
    net.affine_displace(a["miny"], H, 0.01 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-8, criterion="rms", max_steps=200000, **FIRE))
    assert rep.status == nr.NR_OK and rep.e_gel > 0
    x = net.positions()
    F = net.forces()
    i, j = a["mpairs"][:, 0], a["mpairs"][:, 1]
    assert np.array_equal(F[i], F[j])
    assert np.abs((x[j, 0] - x[i, 0]) - a["offset"]).max() < 1e-9 and np.array_equal(x[j, 1], x[i, 1])
