"""The parallel .dat reader, the parallel writer, parallel get_triples and
the binary side-car, on the CPU.

The reader must give exactly what read_network gives (the oracle restates
it with getline / sscanf, large_strain_relax.cu:42-114): fuzzed files mix
plain and unusual number forms (signs, exponents, hex floats, '1e', values
out of a char's range, CRLF, NULs, comments, blank and short lines) so the
fast path and its sscanf fallback both run; points, bonds, rest lengths,
wraps, ranges and the accept / reject verdict must be identical.
"""
import os

import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

NUM_FORMS = ["%r", "%.17g", "%+.6f", "%.3e", "%E", "0x1.8p+1", "1e", "%g ", " %r", "%r,", "inf", "-0"]


def _num(rng, v):
    f = NUM_FORMS[rng.integers(len(NUM_FORMS))] if rng.random() < 0.3 else "%r"
    return f % v if "%" in f else f


def _fuzz_file(path, rng, n, m):
    pts = rng.uniform(-5, 5, (n, 2))
    lines = ["%d %d %r" % (n, m, float(rng.uniform(1, 10)))]
    for x, y in pts:
        r = rng.random()
        if r < 0.05:
            lines.append("# comment")
        elif r < 0.08:
            lines.append("")
        lines.append("%s %s%s" % (_num(rng, float(x)), _num(rng, float(y)), " extra" if rng.random() < 0.05 else ""))
    for _ in range(m):
        i, j = rng.integers(-1 if rng.random() < 0.01 else 0, n + (1 if rng.random() < 0.01 else 0), 2)
        w = int(rng.choice([-1, 0, 1, 200, -300])) if rng.random() < 0.05 else int(rng.integers(-1, 2))
        sep = rng.choice([" ", "\t", "  "])
        lines.append("%s%s%s%s%s" % (("+" if rng.random() < 0.05 else "") + str(i), sep, j, sep, w))
        if rng.random() < 0.03:
            lines.append("7 8")
    text = "\n".join(lines)
    if rng.random() < 0.3:
        text = text.replace("\n", "\r\n")
    if rng.random() < 0.5:
        text += "\n"
    if rng.random() < 0.1:
        text = text[: int(len(text) * rng.uniform(0.5, 1.0))]
    data = text.encode()
    if rng.random() < 0.05:
        k = int(rng.integers(len(data)))
        data = data[:k] + b"\0" + data[k:]
    with open(path, "wb") as f:
        f.write(data)


def _same(path):
    ok_o, a = oracle.read_network(path, want_triples=False)
    try:
        h = nr.HostNetwork.read(path, strict=False)
    except nr.NetRelaxError:
        assert len(a["points"]) == 0, path
        return
    b = h.arrays()
    ok_n = True
    try:
        nr.HostNetwork.read(path)
    except nr.NetRelaxError:
        ok_n = False
    assert ok_n == ok_o
    assert np.array_equal(a["points"], b["points"])
    assert np.array_equal(a["edge_ij"], b["edge_ij"]) and np.array_equal(a["edge_wrap"], b["edge_wrap"])
    assert [v.hex() for v in a["edge_l0"]] == [float(v).hex() for v in b["edge_l0"]]
    if len(a["points"]):
        assert a["miny"] == b["miny"] and a["maxy"] == b["maxy"]


@pytest.mark.parametrize("seed", range(40))
def test_reader_matches_read_network_on_fuzzed_files(seed, tmp_path):
    rng = np.random.default_rng(seed)
    path = str(tmp_path / "f.dat")
    _fuzz_file(path, rng, int(rng.integers(1, 60)), int(rng.integers(0, 90)))
    _same(path)


def test_reader_large_file_threads(tmp_path):
    """A 200 x 200 lattice read with 1 and with 8 threads: identical, and
    identical to the oracle."""
    h = nr.HostNetwork.lattice(200, 200, 0.7, 0.05, 3)
    path = str(tmp_path / "big.dat")
    h.write(path)
    os.environ["NR_IO_THREADS"] = "1"
    try:
        a1 = nr.HostNetwork.read(path).get_triples().arrays()
    finally:
        os.environ.pop("NR_IO_THREADS")
    os.environ["NR_IO_THREADS"] = "8"
    try:
        a8 = nr.HostNetwork.read(path).get_triples().arrays()
    finally:
        os.environ.pop("NR_IO_THREADS")
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap"):
        assert np.array_equal(a1[k], a8[k]), k
    _same(path)
    ok, o = oracle.read_network(path)
    assert np.array_equal(o["tri_hjk"], a8["tri_hjk"]) and np.array_equal(o["tri_wrap"], a8["tri_wrap"])


def test_writer_round_trips_and_matches_printf(tmp_path):
    h = nr.HostNetwork.lattice(60, 40, 0.7, 0.1, 5)
    a = h.arrays()
    path = str(tmp_path / "w.dat")
    h.write(path)
    expect = ["%d %d %.17g" % (len(a["points"]), len(a["edge_l0"]), a["offset"])]
    expect += ["%.17g %.17g" % (x, y) for x, y in a["points"]]
    expect += ["%d %d %d" % (i, j, w) for (i, j), w in zip(a["edge_ij"], a["edge_wrap"])]
    assert open(path).read() == "\n".join(expect) + "\n"
    b = nr.HostNetwork.read(path).arrays()
    assert np.array_equal(a["points"], b["points"]) and np.array_equal(a["edge_l0"], b["edge_l0"])


def test_binary_side_car(tmp_path):
    h = nr.HostNetwork.lattice_mesh(30, 20, 0.7, 0.1, 2).get_triples()
    h.set_bond_k(np.linspace(1, 2, h.info().n_edges))
    a = h.arrays()
    path = str(tmp_path / "n.bin")
    h.write_bin(path)
    b = nr.HostNetwork.read_bin(path).arrays()
    for k in ("points", "edge_ij", "edge_l0", "edge_wrap", "tri_hjk", "tri_wrap", "bond_k", "facets", "areas",
              "mpairs"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("offset", "miny", "maxy", "minx", "maxx"):
        assert a[k] == b[k]
    data = bytearray(open(path, "rb").read())
    data[len(data) // 2] ^= 0x40
    open(path, "wb").write(bytes(data))
    for bad in (bytes(data), bytes(data[: len(data) // 3])):
        open(path, "wb").write(bad)
        with pytest.raises(nr.NetRelaxError) as e:
            nr.HostNetwork.read_bin(path)
        assert e.value.status == nr.NR_ERR_PARSE


def test_binary_side_car_rejects_every_damaged_file(tmp_path):
    """Flipped bits anywhere (header fields included), truncation and
    trailing bytes all give NR_ERR_PARSE; a count damaged to billions is
    caught by the file size before anything is allocated."""
    h = nr.HostNetwork.lattice_mesh(12, 9, 0.7, 0.1, 2).get_triples()
    path = str(tmp_path / "n.bin")
    h.write_bin(path)
    good = open(path, "rb").read()
    rng = np.random.default_rng(3)
    for t in range(400):
        data = bytearray(good)
        if t % 3 == 0:
            k = int(rng.integers(len(data))) if t % 2 else int(rng.integers(112))  # 112-byte header
            data[k] ^= int(rng.integers(1, 256))
        elif t % 3 == 1:
            data = data[: int(rng.integers(len(data)))]
        else:
            data += bytes(int(v) for v in rng.integers(0, 256, int(rng.integers(1, 40))))
        open(path, "wb").write(bytes(data))
        with pytest.raises(nr.NetRelaxError) as e:
            nr.HostNetwork.read_bin(path)
        assert e.value.status == nr.NR_ERR_PARSE, t
    data = bytearray(good)
    data[24:32] = (2 ** 31).to_bytes(8, "little")  # n_edges
    open(path, "wb").write(bytes(data))
    with pytest.raises(nr.NetRelaxError) as e:
        nr.HostNetwork.read_bin(path)
    assert e.value.status == nr.NR_ERR_PARSE


def test_positions_writer_matches_report_displaced(tmp_path):
    """"%2.10le\t%2.10le" per node, as report_displaced writes .pos files."""
    rng = np.random.default_rng(4)
    xy = np.ascontiguousarray(np.concatenate([rng.normal(size=(3000, 2)) * 10.0 ** rng.integers(-12, 12, (3000, 2)),
                                              [[0.0, -0.0], [1e-310, -5e-324], [1.0, 99999.999999999]]]))
    path = str(tmp_path / "p.pos")
    nr.check(nr.lib().nr_write_positions(xy.ctypes.data_as(nr.C.POINTER(nr.C.c_double)), len(xy), path.encode()),
             "write_positions")
    assert open(path).read() == "".join("%2.10le\t%2.10le\n" % (x, y) for x, y in xy)


@pytest.mark.parametrize("seed", range(60))
def test_oracle_reader_matches_live_reference_on_fuzzed_files(seed, tmp_path):
    """The oracle's restatement against the reference's own read_network
    (and get_triples) built for the host, on the same fuzzed files."""
    if oracle.build_ref() is None or oracle.ref_lib() is None:
        pytest.skip("reference checkout not available (golden fixtures cover this case)")
    rng = np.random.default_rng(seed)
    path = str(tmp_path / "f.dat")
    _fuzz_file(path, rng, int(rng.integers(1, 60)), int(rng.integers(0, 90)))
    ok_o, a = oracle.read_network(path)
    ok_r, r = oracle.ref_read_network(path)
    assert ok_o == ok_r
    keys = ("points", "edge_ij", "edge_wrap") + (("tri_hjk", "tri_wrap") if ok_o else ())
    for k in keys:
        assert np.array_equal(a[k], r[k]), k
    assert [float(v).hex() for v in a["edge_l0"]] == [float(v).hex() for v in r["edge_l0"]]
    if ok_o:
        assert (a["offset"], a["miny"], a["maxy"]) == (r["offset"], r["miny"], r["maxy"])
