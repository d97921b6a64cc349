"""Gel coupling (network_mesh_relax.cu) on the CPU: the oracle and the host
side of the library against the reference.

Golden fixtures (tests/golden/mesh/, made by the reference's own code with
tests/golden/make_mesh_golden.py) always; the host-compiled reference live
where its checkout exists.  Bars: reader, duplicate pairs, inverse matrices,
dilation and pure-gel forces bit-exact; forces with bonds within 1e-15 of
the largest force (the reference's rhypot against 1/sqrt); relaxations
within 1e-12 of the total energy per term and 1e-10 in position; the sweep within
the 9 significant digits the reference's edata file prints.
"""
import json
import math
import os

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "mesh")
FIRE = [0.1, 0.99, 0.1, 1.1, 0.5]
GEL = dict(smod=0.7, bmod=2.0, dilation=0.05)
FORCE_CASES = [(0.0, 0.0), (1.0, 0.0), (1.0, 1e-2)]


def _readers():
    return json.load(open(os.path.join(GOLD, "ref_readers.json")))


def _unhex(v):
    return np.array([float.fromhex(x) for x in v])


def _assert_reader(name, ok, a, r, with_triples=True):
    assert ok == r["ok"], name
    assert np.array_equal(a["points"].reshape(-1), _unhex(r["points"])), name
    assert np.array_equal(a["edge_l0"], _unhex(r["edge_l0"])), name
    assert np.array_equal(a["areas"], _unhex(r["areas"])), name
    for k in ("edge_ij", "edge_wrap", "facets", "mpairs") + (("tri_hjk", "tri_wrap") if with_triples else ()):
        assert np.asarray(a[k]).reshape(-1).tolist() == r[k], (name, k)
    if r["ok"]:
        for k in ("offset", "minx", "miny", "maxx", "maxy"):
            assert float(a[k]).hex() == r[k], (name, k)


def _fcodes(a):
    y = a["points"][:, 1]
    return np.where((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10), 0, 3).astype(np.uint8)


def _m1():
    ok, a = oracle.read_network_mesh(os.path.join(GOLD, "m1.nmc"))
    assert ok
    return a, np.load(os.path.join(GOLD, "ref_m1.npz"))


# ---------------------------------------------------------------- readers

def test_oracle_mesh_reader_matches_golden():
    for name, r in _readers().items():
        ok, a = oracle.read_network_mesh(os.path.join(GOLD, name))
        _assert_reader(name, ok, a, r)


def test_library_mesh_reader_matches_golden():
    """nr_read_network_mesh (partial networks returned on parse errors)."""
    for name, r in _readers().items():
        path = os.path.join(GOLD, name)
        try:
            h = nr.HostNetwork.read_mesh(path, strict=False)
        except nr.NetRelaxError:
            assert not r["ok"] and not r["points"], name  # rejected at the header
            continue
        a = h.get_triples().arrays()
        ok = True
        try:
            nr.HostNetwork.read_mesh(path)
        except nr.NetRelaxError as e:
            ok = False
            assert e.status == nr.NR_ERR_PARSE
        _assert_reader(name, ok, a, r)


def test_mesh_writer_round_trips():
    h = nr.HostNetwork.lattice_mesh(9, 7, 0.75, 0.2, seed=4)
    a = h.arrays()
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "nr_roundtrip.nmc")
    h.write_mesh(path)
    b = nr.HostNetwork.read_mesh(path).arrays()
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "facets", "areas", "mpairs"):
        assert np.array_equal(a[k], b[k]), k
    ok, c = oracle.read_network_mesh(path)
    assert ok and np.array_equal(c["mpairs"], a["mpairs"])


def test_generator_layout():
    """Copy column paired with column 0; triangles tile the box; seeded."""
    nx, ny = 8, 6
    a = nr.HostNetwork.lattice_mesh(nx, ny, 0.7, 0.1, seed=9).arrays()
    assert len(a["points"]) == (nx + 1) * ny and len(a["facets"]) == 2 * nx * (ny - 1)
    assert a["mpairs"].tolist() == [[j * (nx + 1), j * (nx + 1) + nx] for j in range(ny)]
    assert abs(a["areas"].sum() - nx * (ny - 1)) < 1e-9
    b = nr.HostNetwork.lattice_mesh(nx, ny, 0.7, 0.1, seed=9).arrays()
    assert all(np.array_equal(a[k], b[k]) for k in ("points", "edge_ij", "facets"))


def test_pair_search_matches_oracle_on_near_duplicates():
    """The library's std::map search and the oracle's sorted-array restatement
    agree on points closer than the 1e-10 tolerance."""
    rng = np.random.default_rng(3)
    for trial in range(20):
        n = 40
        pts = np.column_stack([rng.integers(0, 3, n) * 1.0, rng.integers(0, 6, n) * 0.5])
        pts += rng.choice([0.0, 1e-12, -1e-12, 3e-10], size=pts.shape)
        h = nr.HostNetwork.from_arrays(pts, np.zeros((0, 2)), np.zeros(0), 2.0)
        minx = pts[:, 0].min()
        h.set_mesh(np.zeros((0, 3)), np.zeros(0))
        assert h.arrays()["mpairs"].tolist() == oracle.mesh_pairs(pts, 2.0, minx).tolist(), trial


# ---------------------------------------------------------------- physics

def test_inv_mats_and_dilate_bit_exact():
    a, g = _m1()
    assert np.array_equal(oracle.inv_mats(a["points"], a["facets"]), g["inv_mats"])
    x = g["x_pert"]
    if oracle.ref_mesh_lib() is not None:
        assert np.array_equal(oracle.dilate(x, 0.0, 0.0, 1.1), oracle.ref_dilate(x, 0.0, 0.0, 1.1))


def test_gel_forces_match_golden():
    a, g = _m1()
    gel = oracle.mesh_gel(a, inv=g["inv_mats"], **GEL)
    for c, (ks, kb) in enumerate(FORCE_CASES):
        m = oracle.Model(a, ks, kb, fcodes=g["fcodes"], gel=gel)
        F = m.forces(g["x_pert"])
        ref = g["forces_%d" % c]
        if ks == 0 and kb == 0:
            assert np.array_equal(F, ref)  # gel_forces + duplicate_forces, serialised
        else:
            assert np.abs(F - ref).max() <= 1e-15 * np.abs(ref).max()
    # duplicate vertices carry the same force
    for i, j in a["mpairs"]:
        assert np.array_equal(F[i], F[j])


def test_gel_energy_matches_golden():
    a, g = _m1()
    m = oracle.Model(a, 1.0, 0.0, fcodes=g["fcodes"], gel=oracle.mesh_gel(a, inv=g["inv_mats"], **GEL))
    ref = np.abs(g["gel_energies"]).sum()
    assert abs(m.gel_energy(g["x_pert"]) - ref) <= 1e-14 * ref


def test_fire_matches_golden_reference_run():
    a, g = _m1()
    m = oracle.Model(a, 1.0, 1e-2, fcodes=g["fcodes"], gel=oracle.mesh_gel(a, inv=g["inv_mats"], **GEL))
    x, v, F, rep = m.fire(g["x_affine"], oracle.params(fcut=1e-9, criterion="rms", max_steps=200000))
    r = g["fire_report"]
    assert rep.steps == int(g["fire_steps"])
    total = sum(r[1:])
    for mine, theirs in zip((rep.e_stretch, rep.e_bend, rep.e_gel), r[1:]):
        assert abs(mine - theirs) <= 1e-12 * total
    assert abs(rep.rms_force - r[0]) <= 1e-3 * r[0]
    assert np.abs(x - g["fire_pos"]).max() < 1e-10


def _oracle_protocol(path, prm):
    """network_mesh_relax.cu:1095-1376 on the oracle: (records, positions)."""
    s = math.sqrt(1 + prm["dilation"])
    ok, a = oracle.read_network_mesh(path)
    ok, a = oracle.read_network_mesh(path, triple_offset=a["offset"] * s)
    assert ok
    fc = _fcodes(a)
    inv = oracle.inv_mats(a["points"], a["facets"])
    x = oracle.dilate(a["points"], a["minx"], a["miny"], s)
    a2 = dict(a)
    a2["offset"] = a["offset"] * s
    es, _ = oracle.Model(a2, prm["ks"], prm["kb"], fcodes=fc).energies(x)
    area = (a["maxx"] - a["minx"]) * (a["maxy"] - a["miny"])
    pref = oracle.preferred_dilation(prm["ks"], es, area, prm["dilation"], prm["bmod"])
    gel = oracle.mesh_gel(a, prm["smod"], prm["bmod"], pref, inv=inv)
    m = oracle.Model(a2, prm["ks"], prm["kb"], fcodes=fc, gel=gel)
    p = oracle.params(*prm["fire"], nmin=prm["nmin"], mass=prm["mass"], fcut=prm["fcut"], max_steps=prm["nmax"],
                      criterion="rms")
    recs, shp, _ = m.mesh_sweep(x, a["miny"], (a["maxy"] - a["miny"]) * s, p, prm["compr"], prm["shear"])
    return recs, shp, pref


def test_sweep_matches_golden_reference_run():
    d = os.path.join(GOLD, "ref_sweep")
    prm = json.load(open(os.path.join(d, "params.json")))
    recs, shp, _ = _oracle_protocol(os.path.join(GOLD, "sweep.nmc"), prm)
    ref = np.loadtxt(os.path.join(d, "sweep_edata.txt"))
    assert len(recs) == len(ref)
    mine = np.array([[r[0], r[1], r[2], r[3], r[4], r[2] + r[3] + r[4]] for r in recs])
    assert np.allclose(mine, ref, rtol=2e-8, atol=1e-8)
    steps = [int(ln.split("Steps: ")[1].split(",")[0]) for ln in open(os.path.join(d, "sweep_log.txt"))]
    assert [int(r[7]) for r in recs] == steps
    shear_rows = [k for k, r in enumerate(recs) if r[8] == 1]
    for n, k in enumerate(shear_rows):
        P = np.loadtxt(os.path.join(d, "sweep_%d.pos" % (n + 1)))
        assert np.abs(P - shp[k]).max() < 1e-8


def test_mesh_batch_parser_matches_golden():
    ref = json.load(open(os.path.join(GOLD, "ref_batch.json")))
    for name, r in ref.items():
        path = os.path.join(GOLD, "batch_files", name)
        try:
            s = nr.parse_mesh_batch_file(path)
        except nr.NetRelaxError:
            assert not r["ok"], name
            continue
        assert r["ok"], name
        assert s.net.base.decode() == r["base"] and s.net.tag.decode() == r["tag"]
        assert [s.net.ks, s.net.kb, s.bmod, s.smod, s.dilation] == r["mech"]
        assert list(s.net.fire_params) == r["fire"] and list(s.net.compr) == r["compr"]
        assert list(s.net.shear) == r["shear"]
        assert (s.net.nmin, s.net.mass, s.net.fcut, s.net.nmax) == (r["nmin"], r["mass"], r["fcut"], r["nmax"])


# ---------------------------------------------------------------- live reference

def _need_ref():
    if oracle.ref_mesh_lib() is None and (oracle.build_ref() is None or oracle.ref_mesh_lib() is None):
        pytest.skip("reference checkout not present")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_live_reference_random_meshes(seed, tmp_path):
    _need_ref()
    rng = np.random.default_rng(seed)
    nx, ny = int(rng.integers(4, 14)), int(rng.integers(3, 10))
    path = str(tmp_path / "r.nmc")
    nr.HostNetwork.lattice_mesh(nx, ny, float(rng.uniform(0.4, 1.0)), float(rng.uniform(0, 0.2)),
                                seed=seed).write_mesh(path)
    ok, a = oracle.read_network_mesh(path)
    ok2, r = oracle.ref_read_network_mesh(path)
    assert ok and ok2
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap", "facets", "areas", "mpairs"):
        assert np.array_equal(a[k], r[k]), k
    fc = _fcodes(a)
    gel = oracle.mesh_gel(a, float(rng.uniform(0.1, 2)), float(rng.uniform(0.1, 3)), float(rng.uniform(0, 0.2)))
    x = a["points"] + rng.normal(0, 0.05, a["points"].shape) * (fc[:, None] > 0)
    for i, j in a["mpairs"]:
        x[j] = x[i] + [a["offset"], 0.0]
    F = oracle.Model(a, 0.0, 0.0, fcodes=fc, gel=gel).forces(x)
    assert np.array_equal(F, oracle.ref_mesh_forces(a, x, a["offset"], 0.0, 0.0, gel, fc))


# ------------------------------------------------------ fuzzed .nmc files

def _fuzz_mesh(path, rng):
    """A generated composite written as .nmc, then mutated line by line:
    dropped, duplicated or junk lines (so lines shift between sections and
    are parsed as the next section's), tabs, trailing fields, CRLF, negative
    areas, out-of-range indices, wraps outside a char's range, truncation."""
    src = path + ".src"
    nr.HostNetwork.lattice_mesh(int(rng.integers(3, 8)), int(rng.integers(3, 6)), float(rng.uniform(0.5, 1.0)),
                                float(rng.uniform(0, 0.2)), seed=int(rng.integers(1, 1000))).write_mesh(src)
    lines = open(src).read().split("\n")
    os.remove(src)
    n = int(lines[0].split()[0])
    out = [lines[0]]
    for ln in lines[1:]:
        r = rng.random()
        if r < 0.002:
            continue
        if r < 0.004:
            out.append(ln)
        elif r < 0.02:
            out.append("# junk")
        elif r < 0.04:
            out.append("")
        f = ln.split()
        if f and rng.random() < 0.004:
            if len(f) == 1:
                f[0] = rng.choice(["-1.5", "0", "1e-300", "0x1p-2"])
            elif len(f) == 3 and "." not in ln:
                k = int(rng.integers(3))
                f[k] = str(rng.choice([-1, n, n + 5, 200, -300]))
            ln = rng.choice([" ", "\t", "  "]).join(f)
        if rng.random() < 0.01:
            ln += " 7"
        out.append(ln)
    text = "\n".join(out)
    if rng.random() < 0.3:
        text = text.replace("\n", "\r\n")
    if rng.random() < 0.15:
        text = text[: int(len(text) * rng.uniform(0.3, 1.0))]
    with open(path, "w") as fh:
        fh.write(text)


def _same_mesh(a, b, ok_a, ok_b, label, triples=False):
    assert ok_a == ok_b, label
    for k in ("points", "edge_ij", "edge_wrap", "facets", "areas", "mpairs") + (("tri_hjk", "tri_wrap") if triples
                                                                                 else ()):
        assert np.array_equal(np.asarray(a[k]).reshape(-1), np.asarray(b[k]).reshape(-1)), (label, k)
    assert [float(v).hex() for v in a["edge_l0"]] == [float(v).hex() for v in b["edge_l0"]], label
    if ok_a:
        for k in ("offset", "minx", "miny", "maxx", "maxy"):
            assert float(a[k]).hex() == float(b[k]).hex(), (label, k)


@pytest.mark.parametrize("seed", range(60))
def test_mesh_reader_on_fuzzed_files(seed, tmp_path):
    """nr_read_network_mesh returns what the oracle's restatement of
    read_network_mesh does, accept / reject verdict and partial arrays
    included."""
    rng = np.random.default_rng(1000 + seed)
    path = str(tmp_path / "f.nmc")
    _fuzz_mesh(path, rng)
    ok_o, a = oracle.read_network_mesh(path)
    try:
        h = nr.HostNetwork.read_mesh(path, strict=False)
    except nr.NetRelaxError:
        assert not ok_o and len(a["points"]) == 0, path
        return
    b = dict(h.arrays())
    b.update(minx=h.mesh_info().minx, maxx=h.mesh_info().maxx)
    ok_n = True
    try:
        nr.HostNetwork.read_mesh(path)
    except nr.NetRelaxError:
        ok_n = False
    _same_mesh(a, b, ok_o, ok_n, "seed %d" % seed)


@pytest.mark.parametrize("seed", range(20))
def test_live_reference_mesh_reader_on_fuzzed_files(seed, tmp_path):
    """The oracle's reader against the reference's own read_network_mesh
    (and get_triples) on the same fuzzed files."""
    _need_ref()
    rng = np.random.default_rng(1000 + seed)
    path = str(tmp_path / "f.nmc")
    _fuzz_mesh(path, rng)
    ok_o, a = oracle.read_network_mesh(path)
    ok_r, r = oracle.ref_read_network_mesh(path)
    _same_mesh(a, r, ok_o, ok_r, "seed %d" % seed, triples=ok_o and ok_r)
