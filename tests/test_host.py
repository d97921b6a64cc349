"""Host side of the library (no GPU): reader, triple finder, generators,
batch files, file lists, the C ABI's exports and error behaviour."""
import ctypes as C
import json
import os
import re
import subprocess
import sys

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
    assert lib.nr_abi_version() == 2
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


def _fuzz_batch(path, rng, kind):
    """A batch file of one of the three grammars (lsrelax, nmrelax,
    sp_relax) with random values and the mistakes users make: comments,
    blank lines, tabs, CRLF (often with a space before the CR), too few or
    non-numeric values, negative values, reversed ranges, NUL bytes inside
    a line, truncation.  sp_relax files are never truncated: the
    reference's parser returns an uninitialised flag when the file ends
    before the shear line, so their entry lines are never empty either."""

    def num(lo, hi):
        v = float(rng.uniform(lo, hi))
        return rng.choice(["%r" % v, "%.3g" % v, "%d" % int(v), "%.2e" % v])

    def vals(k, lo, hi, ordered=False):
        if rng.random() < 0.85:
            lo = 0.0  # mostly valid values, so that accepted files are common too
        x = [float(rng.uniform(lo, hi)) for _ in range(k)]
        if ordered and rng.random() < 0.9:
            x[:2] = sorted(x[:2])
        out = [rng.choice(["%r" % v, "%.3g" % v, "%d" % int(v), "%.2e" % v]) for v in x]
        if rng.random() < 0.1:
            out.insert(int(rng.integers(len(out) + 1)), rng.choice(["abc", "1e", "0x10", "nan", "-"]))
        if rng.random() < 0.08:
            out = out[: int(rng.integers(len(out) + 1))]
        return rng.choice([" ", "\t", "  "]).join(out)

    base = rng.choice(["nets/lat", "a", "./x_y", "dir/sub/net"]) + (" tag%d" % rng.integers(9) if rng.random() < 0.5
                                                                     else "")
    if kind == "spr":
        # An empty entry line would shift the later entries up and leave the
        # shear line missing: a junk line stands in for it.
        lines = [base] + [vals(3, lo, hi, o) or "x" for lo, hi, o in ((-0.2, 3, False), (-0.01, 0.2, True),
                                                                       (-0.01, 0.2, True))]
    else:
        lines = [base, vals(2 if kind == "lsr" else int(rng.integers(2, 6)), -0.2, 3),
                 vals(int(rng.integers(4, 9)), -0.1, 2),
                 "%d %s %s %d" % (rng.integers(-2, 8), num(-0.02, 2), num(-1e-10, 1e-8), rng.integers(-5, 10 ** 6)),
                 vals(3, -0.01, 0.2, True), vals(3, -0.01, 0.2, True)]
        if rng.random() < 0.1:
            lines[3] = " ".join(lines[3].split()[: int(rng.integers(4))])
    crlf = rng.random() < 0.3
    out = []
    for ln in lines:
        while rng.random() < 0.2:
            out.append(rng.choice(["# comment", "", "#"]))
        if rng.random() < (0.4 if crlf else 0.1):
            ln += " "
        if rng.random() < 0.05 and len(ln) > 2:
            k = int(rng.integers(1, len(ln)))
            ln = ln[:k] + "\0" + ln[k:]
        out.append(ln)
    text = "\n".join(out) + ("\n" if rng.random() < 0.7 else "")
    if crlf:
        text = text.replace("\n", "\r\n")
    if kind != "spr" and rng.random() < 0.1:
        text = text[: int(len(text) * rng.uniform(0.5, 1.0))]
    with open(path, "wb") as f:
        f.write(text.encode())


def _ref_parse(kind, path):
    """The reference's own parse_batch_file of that grammar: (ok, values)."""
    base, tag = C.create_string_buffer(1024), C.create_string_buffer(256)
    fp, cr, sh = (C.c_double * 5)(), (C.c_double * 3)(), (C.c_double * 3)()
    mass, fcut, nmin, nmax = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    if kind == "spr":
        mech = (C.c_double * 3)()
        ok = oracle.ref_spr_lib().ref_spr_parse_batch_file(path.encode(), base, 1024, tag, 256, mech, cr, sh)
        return bool(ok), (base.value, tag.value, list(mech), list(cr), list(sh))
    if kind == "nmr":
        mech = (C.c_double * 5)()
        ok = oracle.ref_mesh_lib().ref_mesh_parse_batch_file(path.encode(), base, 1024, tag, 256, mech, fp,
                                                             C.byref(nmin), C.byref(mass), C.byref(fcut),
                                                             C.byref(nmax), cr, sh)
    else:
        ks, kb = C.c_double(), C.c_double()
        ok = oracle.ref_lib().ref_parse_batch_file(path.encode(), base, 1024, tag, 256, C.byref(ks), C.byref(kb),
                                                   fp, C.byref(nmin), C.byref(mass), C.byref(fcut), C.byref(nmax),
                                                   cr, sh)
        mech = [ks.value, kb.value]
    return bool(ok), (base.value, tag.value, list(mech), list(fp), nmin.value, mass.value, fcut.value, nmax.value,
                      list(cr), list(sh))


def _lib_parse(kind, path):
    if kind == "spr":
        s = nr.parse_spr_batch_file(path)
        return (s.base, s.tag, [s.ks, s.kb, s.mu], list(s.compr), list(s.shear))
    if kind == "nmr":
        m = nr.parse_mesh_batch_file(path)
        s, mech = m.net, [m.net.ks, m.net.kb, m.bmod, m.smod, m.dilation]
    else:
        s = nr.parse_batch_file(path)
        mech = [s.ks, s.kb]
    return (s.base, s.tag, mech, list(s.fire_params), s.nmin, s.mass, s.fcut, s.nmax, list(s.compr), list(s.shear))


@pytest.mark.parametrize("kind", ["lsr", "nmr", "spr"])
@pytest.mark.parametrize("seed", range(120))
def test_parse_batch_file_on_fuzzed_files_matches_live_reference(built, tmp_path, kind, seed):
    """The three batch-file parsers against the reference's own, verdict and
    values, on fuzzed files."""
    if oracle.build_ref() is None or oracle.ref_lib() is None:
        pytest.skip("reference checkout not available (golden fixtures cover this case)")
    rng = np.random.default_rng(seed)
    path = str(tmp_path / "batch.txt")
    _fuzz_batch(path, rng, kind)
    ok_r, r = _ref_parse(kind, path)
    try:
        got = _lib_parse(kind, path)
    except nr.NetRelaxError:
        assert not ok_r, open(path, "rb").read()
        return
    assert ok_r, open(path, "rb").read()
    assert repr(got) == repr(r), open(path, "rb").read()


_REF_MAIN = """
import ctypes as C, sys
sys.path.insert(0, %r)
import oracle
args = [a.encode() for a in sys.argv[1:]]
rc = getattr(oracle, sys.argv[1])().%s(len(args) - 1, (C.c_char_p * (len(args) - 1))(*args[1:]))
sys.exit(rc & 255)
"""


@pytest.mark.parametrize("args", ["", "-b", "-b/nonexistent", "-ib /nonexistent", "-x abc -b /nonexistent",
                                  "-x0 -b /nonexistent", "-x 64 -b /nonexistent", "-z -b /nonexistent",
                                  "-- -b /nonexistent", "extra -b /nonexistent", "-y -b /nonexistent",
                                  "-b /nonexistent -x", "-i -x 3 -y 2 -b /nonexistent"])
@pytest.mark.parametrize("prog", ["lsrelax", "nmrelax"])
def test_lsrelax_options_match_the_reference_main(built, args, prog):
    """Option scanning as the reference's getopt loops (large_strain_relax.cu:
    1055, network_mesh_relax.cu:1432): grouped flags, attached arguments,
    '--', operands, and the same messages.  The one difference is the exit
    status after a failed batch: 1 here, 0 in the reference."""
    if oracle.build_ref() is None or oracle.ref_lib() is None or oracle.ref_mesh_lib() is None:
        pytest.skip("reference checkout not available")
    exe = os.path.join(ROOT, "network_relaxation_gb300", prog)
    entry, lib = ("ref_lsrelax_main", "ref_lib") if prog == "lsrelax" else ("ref_nmrelax_main", "ref_mesh_lib")
    mine = subprocess.run([prog] + args.split(), executable=exe, capture_output=True, text=True, timeout=60)
    ref = subprocess.run([sys.executable, "-c", _REF_MAIN % (ROOT, entry), lib, prog] + args.split(),
                         capture_output=True, text=True, timeout=60)
    assert (mine.stdout, mine.stderr) == (ref.stdout, ref.stderr)
    assert mine.returncode == ref.returncode or (ref.returncode == 0 and mine.returncode == 1)


@pytest.mark.parametrize("args", ["-b", "-b/nonexistent", "-sz -b /nonexistent", "-q -b /nonexistent",
                                  "-gn -ib /nonexistent", "op -s -b /nonexistent"])
def test_sp_relax_options_match_the_reference_main(built, args):
    """sparse_relax.cpp's getopt loop (:1177), batch mode only (without -b
    the reference asks questions on standard input)."""
    if oracle.build_ref() is None or oracle.ref_spr_lib() is None:
        pytest.skip("reference checkout not available")
    exe = os.path.join(ROOT, "network_relaxation_gb300", "sp_relax")
    mine = subprocess.run(["sp_relax"] + args.split(), executable=exe, capture_output=True, text=True, timeout=60)
    ref = subprocess.run([sys.executable, "-c", _REF_MAIN % (ROOT, "ref_spr_main"), "ref_spr_lib", "sp_relax"]
                         + args.split(), capture_output=True, text=True, timeout=60, stdin=subprocess.DEVNULL)
    assert (mine.stdout, mine.stderr) == (ref.stdout, ref.stderr)
    assert mine.returncode == ref.returncode or (ref.returncode == 0 and mine.returncode == 1)
