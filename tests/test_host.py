"""Host side of the library (no GPU): reader, triple finder, generators,
batch files, file lists, the C ABI's exports and error behaviour."""
import ctypes as C
import json
import os
import re
import subprocess

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def test_library_exports_every_header_symbol(built):
    header = open(os.path.join(ROOT, "include", "netrelax.h")).read()
    names = set(re.findall(r"\b(nr_[a-z0-9_]+)\s*\(", header))
    lib = nr.lib()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.nr_abi_version() == 1
    out = subprocess.run(["nm", "-D", "--defined-only", nr._capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (nr_[a-z0-9_]+)", out))
    assert names <= exported


def test_reader_matches_golden_reference(built):
    g = np.load(os.path.join(GOLD, "ref_c1.npz"))
    h = nr.HostNetwork.read(os.path.join(GOLD, "c1.dat")).get_triples()
    a = h.arrays()
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a[k], g[k]), k
    assert np.array_equal(h.fcodes(), g["fcodes"])


def test_reader_edge_cases(built):
    ref = json.load(open(os.path.join(GOLD, "ref_readers.json")))
    for name, r in ref.items():
        path = os.path.join(GOLD, "edge_cases", name)
        if r["ok"]:
            a = nr.HostNetwork.read(path).get_triples().arrays()
        else:
            with pytest.raises(nr.NetRelaxError) as e:
                nr.HostNetwork.read(path)
            assert e.value.status == nr.NR_ERR_PARSE
            if r["n_points"] == 0:
                continue
            a = nr.HostNetwork.read(path, strict=False).get_triples().arrays()
        assert a["points"].tolist() == r["points"], name
        assert a["edge_ij"].tolist() == r["edge_ij"], name
        assert [float(v).hex() for v in a["edge_l0"]] == r["edge_l0"], name
        assert a["tri_hjk"].tolist() == r["tri_hjk"] and a["tri_wrap"].tolist() == r["tri_wrap"], name
        assert float(a["miny"]).hex() == r["miny"] and float(a["maxy"]).hex() == r["maxy"], name


def test_reader_missing_file(built):
    with pytest.raises(nr.NetRelaxError) as e:
        nr.HostNetwork.read("/nonexistent/net.dat")
    assert e.value.status == nr.NR_ERR_IO


@pytest.mark.parametrize("n,p,seed", [(9, 0.7, 1), (32, 0.65, 1), (17, 0.55, 8)])
def test_triples_match_oracle(built, tmp_path, n, p, seed):
    h = nr.HostNetwork.lattice(n, n, p, 0.0, seed)
    path = str(tmp_path / "x.dat")
    h.write(path)
    a = nr.HostNetwork.read(path).get_triples().arrays()
    ok, o = oracle.read_network(path)
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a[k], o[k]), k
    # the in-memory generator output is the same network as its .dat round trip
    g = h.get_triples().arrays()
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a[k], g[k]), k


def test_generator_is_deterministic_and_well_formed(built):
    a1 = nr.HostNetwork.lattice(40, 30, 0.65, 0.05, 123, line_triples=True).arrays()
    a2 = nr.HostNetwork.lattice(40, 30, 0.65, 0.05, 123, line_triples=True).arrays()
    for k in ("points", "edge_ij", "edge_l0", "tri_hjk", "tri_phi0"):
        assert np.array_equal(a1[k], a2[k])
    a3 = nr.HostNetwork.lattice(40, 30, 0.65, 0.05, 124, line_triples=True).arrays()
    assert not np.array_equal(a1["edge_ij"], a3["edge_ij"])
    N = 1200
    assert a1["points"].shape == (N, 2)
    E = len(a1["edge_l0"])
    assert abs(E / (3 * N) - 0.65) < 0.05
    # x-periodic wrap: every bond is short in the minimum image
    p = a1["points"]
    dx = p[a1["edge_ij"][:, 1], 0] + a1["offset"] * a1["edge_wrap"] - p[a1["edge_ij"][:, 0], 0]
    dy = p[a1["edge_ij"][:, 1], 1] - p[a1["edge_ij"][:, 0], 1]
    assert np.abs(np.hypot(dx, dy) - 1).max() < 0.2
    # top and bottom rows stay exactly level (clamped by the fcode rule)
    fc = nr.HostNetwork.lattice(40, 30, 0.65, 0.05, 123).fcodes()
    assert (fc == 0).sum() == 80
    # line triples: arms antiparallel-ish at rest, phi0 small
    assert np.abs(a1["tri_phi0"]).max() < 0.3


def test_unjittered_line_triples_equal_reference_triple_set(built):
    """Generator triples (set) == get_triples' set on an exact lattice."""
    h = nr.HostNetwork.lattice(14, 14, 0.7, 0.0, 5, line_triples=True)
    gen = h.arrays()
    ref = nr.HostNetwork.lattice(14, 14, 0.7, 0.0, 5).get_triples().arrays()

    def key(hjk, w):
        out = set()
        for (hh, j, k), (wj, wk) in zip(hjk, w):
            out.add((hh, min((j, wj), (k, wk)), max((j, wj), (k, wk))))
        return out

    assert key(gen["tri_hjk"], gen["tri_wrap"]) == key(ref["tri_hjk"], ref["tri_wrap"])
    assert np.abs(gen["tri_phi0"]).max() < 1e-14


def test_parse_batch_file_matches_reference(built):
    ref = json.load(open(os.path.join(GOLD, "ref_batch.json")))
    for name, r in ref.items():
        path = os.path.join(GOLD, "batch_files", name)
        if not r["ok"]:
            with pytest.raises(nr.NetRelaxError):
                nr.parse_batch_file(path)
            continue
        s = nr.parse_batch_file(path)
        assert s.base.decode() == r["base"] and s.tag.decode() == r["tag"]
        assert (s.ks, s.kb, s.nmin, s.mass, s.fcut, s.nmax) == (r["ks"], r["kb"], r["nmin"], r["mass"], r["fcut"],
                                                                r["nmax"])
        assert list(s.fire_params) == r["fire"] and list(s.compr) == r["compr"] and list(s.shear) == r["shear"]


def test_file_lists(built, tmp_path):
    for name in ("netB.dat", "netA.dat", "other.dat", "netC.txt"):
        (tmp_path / name).write_text("1 0 1\n0 0\n")
    os.mkdir(tmp_path / "netD.dat")
    lists = nr.get_file_lists(str(tmp_path / "net"), "dat", "t1")
    d = str(tmp_path) + "/"
    assert lists == [(d + "netA.dat", d + "netA_t1_log.txt", d + "netA_t1", d + "netA_t1_edata.txt"),
                     (d + "netB.dat", d + "netB_t1_log.txt", d + "netB_t1", d + "netB_t1_edata.txt")]
    assert len(nr.get_file_lists(str(tmp_path) + "/*", "dat")) == 3


def test_invalid_arguments_are_errors_not_crashes(built):
    lib = nr.lib()
    out = C.c_void_p()
    assert lib.nr_gen_lattice(1, 5, 0.5, 0.0, 1, 0, C.byref(out)) == nr.NR_ERR_INVALID
    assert lib.nr_gen_lattice(5, 5, 1.5, 0.0, 1, 0, C.byref(out)) == nr.NR_ERR_INVALID
    pts = np.zeros((3, 2))
    ij = np.array([[0, 5]], np.int32)
    w = np.zeros(1, np.int8)
    with pytest.raises(nr.NetRelaxError):
        nr.HostNetwork.from_arrays(pts, ij, w, 1.0)
    assert lib.nr_relax(None, None, None, None) == nr.NR_ERR_INVALID
    for fn in (lib.nr_sweep, lib.nr_sweep_graph):
        assert fn(None, 0.0, 1.0, None, None, None, None, 0, None, None, None) == nr.NR_ERR_INVALID
    assert "invalid" in lib.nr_status_string(nr.NR_ERR_INVALID).decode()


def test_lsrelax_cli_usage_errors(built):
    exe = os.path.join(ROOT, "network_relaxation_gb300", "lsrelax")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode != 0 and "No batch file was specified" in r.stderr
    r = subprocess.run([exe, "-b", "/nonexistent/batch.txt"], capture_output=True, text=True)
    assert r.returncode != 0 and "could not be read" in r.stderr
