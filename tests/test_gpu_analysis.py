"""Post-relaxation analyses on the GPU (nr_bond_strains,
nr_linear_axial_energy, nr_nonaffinity) against the oracle: per-item
arithmetic as written and the canonical summation tree, so bit-equal."""
import ctypes as C
import os

import numpy as np
import pytest

import network_relaxation_gb300 as nr
from network_relaxation_gb300 import _capi
import oracle

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


def cases():
    a = nr.HostNetwork.read(os.path.join(G, "small.dat")).arrays()
    yield a, np.loadtxt(os.path.join(G, "analysis", "small_disp.txt"))
    b = nr.HostNetwork.lattice(96, 96, 0.7, 0.05, 9).arrays()
    yield b, np.random.default_rng(3).normal(scale=0.02, size=b["points"].shape)


def test_analyses_host_arrays_bitwise(cuda):
    for a, disp in cases():
        edges = (a["edge_ij"], a["edge_wrap"])
        s = nr.get_strains(a["points"], edges, a["offset"], disp)
        assert np.array_equal(s, oracle.bond_strains(a, a["points"], disp))
        for k in (1.0, 2.5):
            assert nr.linear_axial_energy(a["points"], edges, a["offset"], disp, k) == \
                oracle.linear_axial_energy(a, k, a["points"], disp)
        assert nr.calc_na_val(a["points"], disp, a["miny"], -0.01, 0.02) == \
            oracle.nonaffinity(a["points"], disp, a["miny"], -0.01, 0.02)


def test_analyses_device_arrays(cuda):
    import torch

    a, disp = next(cases())
    lib = _capi.load()
    t = lambda x, dt: torch.tensor(np.ascontiguousarray(x), dtype=dt, device="cuda")  # noqa: E731
    p0, u = t(a["points"].ravel(), torch.float64), t(disp.ravel(), torch.float64)
    ij, w = t(a["edge_ij"].ravel(), torch.int32), t(a["edge_wrap"], torch.int8)
    out = torch.empty(len(a["edge_l0"]), dtype=torch.float64, device="cuda")
    vp = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    st = lib.nr_bond_strains(len(a["points"]), len(a["edge_l0"]), a["offset"], vp(p0), vp(u), vp(ij), vp(w), vp(out),
                             None)
    assert st == 0, lib.nr_last_error().decode()
    assert np.array_equal(out.cpu().numpy(), oracle.bond_strains(a, a["points"], disp))
