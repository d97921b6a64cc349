"""nr_energies_noalloc: network energies with no device allocation.

The entry point is for callers that cannot call cudaMalloc or cudaFree: a
host framework that hands out all device memory from its own pool, or a
loop that must not let an allocation synchronize the device.  It keeps its
scratch (per-tile partial sums) in a fixed array inside the library.

Checked through the C ABI against nr_energies (the allocating entry point,
same canonical FP64 sums, so the bar is bit-for-bit equality like the other
FP64 tests) on two calls in a row over different networks: the second call
reuses the scratch array the first one wrote.  Also checks that a size
above the fixed capacity is rejected with NR_ERR_CAPACITY.

The file sorts last, so a failure here comes after every other test ran.
"""
import ctypes as C

import numpy as np
import pytest

import network_relaxation_gb300 as nr
from network_relaxation_gb300 import _capi

pytestmark = pytest.mark.gpu

NR_ERR_CAPACITY = -8
MAX_ITEMS = 4194304  # NR_NOALLOC_MAX_ITEMS


def sheared_network(L, p, seed, ks, kb, gamma):
    """A diluted lattice sheared affinely; returns its host arrays, the
    sheared positions and nr_energies' values for them."""
    h = nr.HostNetwork.lattice(L, L, p, 0.0, seed).get_triples()
    a = h.arrays()
    net = nr.Network(h, ks=ks, kb=kb)
    H = net.maxy - net.miny
    net.affine_displace(net.miny, H, gamma * H, 0.0)
    es, eb = net.energies()
    x = net.positions()
    net.close()
    return a, x, (es, eb)


def device_layout(torch, a, x):
    """The network in the reference's device layout (run_fire_md's arrays)."""
    dev = "cuda"
    return dict(
        pos=torch.tensor(np.ascontiguousarray(x).reshape(-1), dtype=torch.float64, device=dev),
        pairs=torch.tensor(a["edge_ij"].reshape(-1), dtype=torch.int32, device=dev),
        lengths=torch.tensor(a["edge_l0"], dtype=torch.float64, device=dev),
        e_off=torch.tensor(a["edge_wrap"], dtype=torch.int8, device=dev),
        triples=torch.tensor(a["tri_hjk"].reshape(-1), dtype=torch.int32, device=dev),
        t_off=torch.tensor(a["tri_wrap"].reshape(-1), dtype=torch.int8, device=dev),
    )


def call_noalloc(lib, torch, a, t, ks, kb, out, npairs=None):
    vp = lambda tensor: C.c_void_p(tensor.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.nr_energies_noalloc(
        len(a["points"]), len(a["edge_l0"]) if npairs is None else npairs, len(a["tri_hjk"]), a["offset"], ks, kb,
        vp(t["pos"]), vp(t["pairs"]), vp(t["lengths"]), vp(t["e_off"]), vp(t["triples"]), vp(t["t_off"]), vp(out),
        stream)


def test_energies_noalloc_matches_nr_energies_twice(cuda):
    import torch

    lib = _capi.load()
    ks, kb = 1.0, 1e-3
    cases = [sheared_network(40, 0.65, 11, ks, kb, 0.05), sheared_network(24, 0.6, 12, ks, kb, 0.03)]
    # the first call's network has more tiles: stale partials stay behind
    assert len(cases[0][0]["edge_l0"]) > len(cases[1][0]["edge_l0"]) > 0
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    for a, x, (es, eb) in cases:  # two calls in a row
        t = device_layout(torch, a, x)
        assert es > 0 and eb > 0
        st = call_noalloc(lib, torch, a, t, ks, kb, out)
        assert st == 0, lib.nr_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[0] == es and got[1] == eb, (got, es, eb)


def test_energies_noalloc_rejects_oversize(cuda):
    import torch

    lib = _capi.load()
    a, x, _ = sheared_network(8, 0.65, 13, 1.0, 1e-3, 0.01)
    t = device_layout(torch, a, x)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    st = call_noalloc(lib, torch, a, t, 1.0, 1e-3, out, npairs=MAX_ITEMS + 1)
    assert st == NR_ERR_CAPACITY
    assert "capacity" in lib.nr_last_error().decode()


def test_energies_noalloc_bad_index_gives_nan(cuda):
    """A bond index outside [0, n_points) makes the stretch energy NaN (the
    kernel skips the read instead of reading out of bounds); the bend
    energy, from valid triples, is unchanged."""
    import torch

    lib = _capi.load()
    a, x, (es, eb) = sheared_network(16, 0.65, 14, 1.0, 1e-3, 0.02)
    a = dict(a)
    a["edge_ij"] = a["edge_ij"].copy()
    a["edge_ij"][3, 1] = len(a["points"])
    t = device_layout(torch, a, x)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert call_noalloc(lib, torch, a, t, 1.0, 1e-3, out) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.isnan(got[0]) and got[1] == eb


def test_energies_noalloc_zero_stiffness_and_no_triples(cuda):
    """ks <= 0 leaves the stretch term at 0 with the bend term unchanged; a
    network with bonds and no triples (null triple arrays) returns 0."""
    import torch

    lib = _capi.load()
    a, x, (es, eb) = sheared_network(20, 0.65, 15, 1.0, 1e-3, 0.02)
    t = device_layout(torch, a, x)
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    assert call_noalloc(lib, torch, a, t, 0.0, 1e-3, out) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == 0.0 and got[1] == eb
    vp = lambda tensor: C.c_void_p(tensor.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.nr_energies_noalloc(len(a["points"]), len(a["edge_l0"]), 0, a["offset"], 1.0, 1e-3, vp(t["pos"]),
                                 vp(t["pairs"]), vp(t["lengths"]), vp(t["e_off"]), None, None, vp(out), stream)
    assert st == 0, lib.nr_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == es and got[1] == 0.0
