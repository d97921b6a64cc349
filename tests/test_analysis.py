"""Post-relaxation analyses: the oracle restatement pinned against the
reference's own strain_calc and axial_contribution (outputs committed in
tests/golden/analysis/, made by make_analysis_golden.py), against known
answers for calc_na_val, and against the reference's own calc_na_val
(na_calc.cpp built for the host against std stand-ins for its Boost
headers) where the checkout exists."""
import json
import os

import numpy as np

import network_relaxation_gb300 as nr
import oracle

G = os.path.join(os.path.dirname(__file__), "golden")


def small():
    a = nr.HostNetwork.read(os.path.join(G, "small.dat")).arrays()
    disp = np.loadtxt(os.path.join(G, "analysis", "small_disp.txt"))
    return a, disp


def test_strains_match_reference_program(built):
    a, disp = small()
    ours = oracle.bond_strains(a, a["points"], disp)
    ref = np.loadtxt(os.path.join(G, "analysis", "ref_strains.txt"))  # printed with 11 digits
    assert len(ours) == len(ref)
    np.testing.assert_allclose(ours, ref, rtol=6e-11, atol=1e-20)


def test_axial_energy_matches_reference_program(built):
    a, disp = small()
    ref = json.load(open(os.path.join(G, "analysis", "ref_axial.json")))
    for k, e in ref.items():
        assert abs(oracle.linear_axial_energy(a, float(k), a["points"], disp) - e) <= 6e-11 * abs(e)


def test_strains_restate_formula_exactly(built):
    """strain_calc.cpp:108-116 in numpy (no fused operations): bit-equal."""
    a, disp = small()
    P, ij, w = a["points"], a["edge_ij"], a["edge_wrap"].astype(np.float64)
    dxi = (P[ij[:, 1], 0] + w * a["offset"]) - P[ij[:, 0], 0]
    dyi = P[ij[:, 1], 1] - P[ij[:, 0], 1]
    dxf = (dxi + disp[ij[:, 1], 0]) - disp[ij[:, 0], 0]
    dyf = (dyi + disp[ij[:, 1], 1]) - disp[ij[:, 0], 1]
    li, lf = np.sqrt(dxi * dxi + dyi * dyi), np.sqrt(dxf * dxf + dyf * dyf)
    assert np.array_equal(oracle.bond_strains(a, P, disp), (lf - li) / li)


def test_nonaffinity_known_answers(built):
    a, disp = small()
    P, y0 = a["points"], a["miny"]
    aff = np.stack([(P[:, 1] - y0) * 0.03, (P[:, 1] - y0) * -0.02], 1)
    assert oracle.nonaffinity(P, aff, y0, -0.02, 0.03) == 0.0
    shifted = aff + np.array([0.5, -0.25])
    assert oracle.nonaffinity(P, shifted, y0, -0.02, 0.03) == 0.5 * 0.5 + 0.25 * 0.25
    seq = np.mean(((disp[:, 0] - (P[:, 1] - y0) * 0.01) ** 2 + (disp[:, 1] - (P[:, 1] - y0) * 0.0) ** 2))
    assert abs(oracle.nonaffinity(P, disp, y0, 0.0, 0.01) - seq) <= 1e-14 * seq


def test_nonaffinity_matches_reference_calc_na_val(built):
    """The reference's sequential sum, restated in Python, equals its
    calc_na_val bit for bit; the oracle's canonical sum is within 1e-14."""
    import pytest

    if oracle.build_ref() is None or oracle.ref_nonaffinity(np.zeros((1, 2)), np.zeros((1, 2)), 0, 0, 0, 0) is None:
        pytest.skip("reference checkout not available")
    a, disp = small()
    P = a["points"]
    rng = np.random.default_rng(5)
    for axial, shear in ((0.0, 0.01), (-0.02, 0.03), (0.05, 0.0)):
        u = disp + rng.normal(0, 1e-3, disp.shape)
        ref = oracle.ref_nonaffinity(P, u, P[:, 0].min(), a["miny"], axial, shear)
        s = 0.0
        for (x, y), (ux, uy) in zip(P.tolist(), u.tolist()):
            ex, ey = (y - a["miny"]) * shear, (y - a["miny"]) * axial
            s += (ux - ex) * (ux - ex) + (uy - ey) * (uy - ey)
        assert s / len(P) == ref
        assert abs(oracle.nonaffinity(P, u, a["miny"], axial, shear) - ref) <= 1e-14 * ref
