"""Linear response (sparse_relax.cpp) on the GPU vs the oracle.

The solve is an iterative PCG where the reference (and the oracle) solve
directly, so the bar is a tolerance: energies within 1e-9 relative,
displacement fields within 1e-8 of their largest component on full-rank
systems, residuals of every point below 1e-9 of the load; on systems with
floppy modes (CG's minimum-norm solution against a least-squares one) the
energies only.  Against the reference's golden runs, the digits its files
print.
"""
import json
import os
import shutil

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "spr")


def _compare(spr, a, ks, kb, mu, compr, shear, affine, full_rank=True, strain_mode=True):
    recs, fields = oracle.spr_protocol(a, ks, kb, mu, compr, shear, strain_mode=strain_mode, affine=affine)
    assert spr.solve(affine=affine) == nr.NR_OK
    for r, f in zip(recs, fields):
        rec, u = spr.point(r[0], r[1])
        tol = 1e-9 * abs(r[2]) + 1e-20  # energies below 1e-20 are numerical zeros
        assert abs(rec.e_ss - r[3]) <= tol and abs(rec.e_bend - r[4]) <= tol, (r, rec.e_ss)
        if full_rank:
            assert np.abs(u.reshape(-1) - f).max() <= 1e-8 * max(1e-12, np.abs(f).max())
        assert rec.residual <= 1e-9 * max(1.0, np.abs(f).max())


@pytest.mark.parametrize("affine", [True, False])
def test_spr_full_rank_matches_oracle(cuda, affine):
    h = nr.HostNetwork.lattice(12, 10, 0.85, 0.0, 3)
    a = h.arrays()
    spr = nr.Spr(h, 1.0, 1e-2, 0.05)
    _compare(spr, a, 1.0, 1e-2, 0.05, [0.0, 0.02, 0.01], [0.0, 0.03, 0.015], affine)


def test_spr_floppy_energies_match_oracle(cuda):
    """p = 0.65, no bending, no gel: floppy modes beside a loaded rigid
    backbone; energies agree."""
    h = nr.HostNetwork.lattice(12, 10, 0.65, 0.05, 8)
    a = h.arrays()
    spr = nr.Spr(h, 1.0, 0.0, 0.0)
    recs, _ = oracle.spr_protocol(a, 1.0, 0.0, 0.0, [0.0, 0.0, 1.0], [0.0, 0.04, 0.02])
    assert max(r[2] for r in recs) > 1e-6  # the backbone carries load
    _compare(spr, a, 1.0, 0.0, 0.0, [0.0, 0.0, 1.0], [0.0, 0.04, 0.02], True, full_rank=False)


def test_spr_golden_sweeps(cuda):
    for mode in ("affine", "top"):
        d = os.path.join(GOLD, "ref_sweep_" + mode)
        prm = json.load(open(os.path.join(d, "params.json")))
        ok, a = oracle.read_network(os.path.join(GOLD, "s1.dat"))
        spr = nr.Spr(nr.HostNetwork.read(os.path.join(GOLD, "s1.dat")), prm["ks"], prm["kb"], prm["mu"])
        info = spr.info()
        H, W = info.maxy - info.miny, info.maxx - info.minx
        assert spr.solve(affine=bool(prm["affine"])) == nr.NR_OK
        ref = np.loadtxt(os.path.join(d, "energies.txt"))
        k = 0
        c = prm["compr"][0] * H
        while c < prm["compr"][1] * H + 1e-10:
            s = prm["shear"][0] * W
            while s < prm["shear"][1] * W + 1e-10:
                rec, u = spr.point(c, s)
                assert np.allclose([rec.e_ss, rec.e_bend], ref[k, 2:], rtol=2e-10, atol=1e-300), (mode, k)
                disp = np.loadtxt(os.path.join(d, "s1_%d.disp" % (k + 1)))
                assert np.abs(u - disp).max() <= 1e-10 * max(1.0, np.abs(disp).max())
                k += 1
                s += prm["shear"][2] * W
            c += prm["compr"][2] * H
        assert k == len(ref)


def test_sp_relax_cli_matches_golden(cuda, tmp_path):
    d = os.path.join(GOLD, "ref_sweep_affine")
    prm = json.load(open(os.path.join(d, "params.json")))
    shutil.copy(os.path.join(GOLD, "s1.dat"), tmp_path / "s1.dat")
    batch = tmp_path / "batch.txt"
    batch.write_text("%s\n%r %r %r\n%r %r %r\n%r %r %r\n" % (tmp_path / "s1", prm["ks"], prm["kb"], prm["mu"],
                                                           *prm["compr"], *prm["shear"]))
    assert nr.sp_relax_main(["-b", str(batch), "-s", "-i"]) == 0
    mine = np.loadtxt(tmp_path / "s1_edata.txt")
    ref = np.loadtxt(os.path.join(d, "energies.txt"))
    assert mine.shape == ref.shape
    assert np.allclose(mine[:, :2], ref[:, :2], rtol=0, atol=1e-8)
    assert np.allclose(mine[:, 2:], ref[:, 2:], rtol=2e-10, atol=1e-300)
    log = [ln for ln in open(tmp_path / "s1_log.txt") if ln.startswith("Residual")]
    assert len(log) == len(ref) and max(float(ln.split(":")[1]) for ln in log) < 1e-9
    for k in range(len(ref)):
        u = np.loadtxt(tmp_path / ("s1_%d.disp" % (k + 1)))
        assert np.abs(u - np.loadtxt(os.path.join(d, "s1_%d.disp" % (k + 1)))).max() <= 1e-10


def test_spr_large_linearity(cuda):
    """A 300 x 300 lattice (90 000 nodes): the solve converges, residuals stay
    small, and the energy is quadratic in the load: E(2 s) = 4 E(s),
    E(c, 0) + E(0, s) + cross = E(c, s) with the cross term from E(c, -s)."""
    h = nr.HostNetwork.lattice(300, 300, 0.7, 0.05, 9, line_triples=False).get_triples()
    spr = nr.Spr(h, 1.0, 1e-3, 0.01)
    assert spr.solve(affine=True) == nr.NR_OK
    info = spr.info()
    assert max(info.rel_residual) <= 1e-12
    e1, _ = spr.point(0.0, 0.5, want_u=False)
    e2, _ = spr.point(0.0, 1.0, want_u=False)
    assert abs(e2.e_total - 4 * e1.e_total) <= 1e-9 * e2.e_total
    ec, _ = spr.point(0.3, 0.0, want_u=False)
    ecs, _ = spr.point(0.3, 0.5, want_u=False)
    ecm, _ = spr.point(0.3, -0.5, want_u=False)
    assert abs((ecs.e_total + ecm.e_total) - 2 * (ec.e_total + e1.e_total)) <= 1e-9 * ecs.e_total
    assert e2.residual <= 1e-9 * 300
