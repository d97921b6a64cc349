"""Python bindings of the oracle (nr_oracle.c) and of the reference compiled
for the host (oracle/_ref/liblsr_ref.so, present only where the reference
checkout exists).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libnr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "liblsr_ref.so")

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
bp = C.POINTER(C.c_byte)
ubp = C.POINTER(C.c_ubyte)


class OrNet(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_edges", C.c_int), ("n_triples", C.c_int), ("offset", C.c_double),
                ("miny", C.c_double), ("maxy", C.c_double), ("points", dp), ("edge_ij", ip), ("edge_l0", dp),
                ("edge_wrap", bp), ("tri_hjk", ip), ("tri_wrap", bp)]


class OrModel(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_edges", C.c_int), ("n_triples", C.c_int), ("width", C.c_double),
                ("ks", C.c_double), ("kb", C.c_double), ("edge_ij", ip), ("edge_l0", dp), ("edge_wrap", bp),
                ("tri_hjk", ip), ("tri_wrap", bp), ("fcodes", ubp), ("bond_k", dp), ("tri_kb", dp),
                ("tri_phi0", dp)]


class OrParams(C.Structure):
    _fields_ = [("alpha0", C.c_double), ("falpha", C.c_double), ("dt_max", C.c_double), ("finc", C.c_double),
                ("fdec", C.c_double), ("nmin", C.c_int), ("mass", C.c_double), ("fcut", C.c_double),
                ("max_steps", C.c_int), ("criterion", C.c_int)]


class OrReport(C.Structure):
    _fields_ = [("rms_force", C.c_double), ("max_force", C.c_double), ("e_stretch", C.c_double),
                ("e_bend", C.c_double), ("steps", C.c_int), ("converged", C.c_int)]


def build(force=False):
    """Compiles libnr_oracle.so (gcc, seconds)."""
    src = os.path.join(HERE, "nr_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "nr_oracle.h"))):
        subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True)
    return ORACLE_SO


def build_ref():
    """Builds oracle/_ref/liblsr_ref.so when the reference checkout exists."""
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)
    return REF_SO if os.path.exists(REF_SO) else None


_or = None


def lib():
    global _or
    if _or is None:
        build()
        L = C.CDLL(ORACLE_SO)
        L.or_read_network.argtypes = [C.c_char_p, C.POINTER(OrNet)]
        L.or_get_triples.argtypes = [C.POINTER(OrNet)]
        L.or_free_net.argtypes = [C.POINTER(OrNet)]
        L.or_fcodes.argtypes = [C.POINTER(OrNet), dp, ubp]
        L.or_affine_displace.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.or_atan2.restype = C.c_double
        L.or_atan2.argtypes = [C.c_double, C.c_double]
        L.or_canon_sum.restype = C.c_double
        L.or_canon_sum.argtypes = [dp, C.c_long]
        L.or_bond_strains.argtypes = [C.c_int, ip, bp, C.c_double, dp, dp, dp]
        L.or_linear_axial_energy.restype = C.c_double
        L.or_linear_axial_energy.argtypes = [C.c_int, ip, bp, C.c_double, C.c_double, dp, dp]
        L.or_nonaffinity.restype = C.c_double
        L.or_nonaffinity.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.c_double]
        L.or_forces.argtypes = [C.POINTER(OrModel), dp, dp]
        L.or_energies.argtypes = [C.POINTER(OrModel), dp, dp, dp]
        L.or_fire.argtypes = [C.POINTER(OrModel), dp, dp, dp, C.POINTER(OrParams), C.POINTER(OrReport)]
        L.or_sweep.restype = C.c_int
        L.or_sweep.argtypes = [C.POINTER(OrModel), dp, C.c_double, C.c_double, C.POINTER(OrParams), dp, dp, dp,
                               C.c_int, dp]
        L.or_fire_batch.argtypes = [C.c_int, C.POINTER(OrModel), C.POINTER(dp), C.POINTER(OrParams),
                                    C.POINTER(OrReport), C.c_int]
        _or = L
    return _or


def _d(a):
    return a.ctypes.data_as(dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(ip)


def _b(a):
    return a.ctypes.data_as(bp)


def read_network(path, want_triples=True):
    """or_read_network + or_get_triples -> (ok, dict of numpy arrays)."""
    L = lib()
    net = OrNet()
    ok = L.or_read_network(str(path).encode(), C.byref(net))
    if want_triples and net.points:
        L.or_get_triples(C.byref(net))
    out = {
        "offset": net.offset, "miny": net.miny, "maxy": net.maxy,
        "points": np.ctypeslib.as_array(net.points, (net.n_points, 2)).copy() if net.n_points else np.zeros((0, 2)),
        "edge_ij": np.ctypeslib.as_array(net.edge_ij, (net.n_edges, 2)).copy() if net.n_edges else np.zeros((0, 2), np.int32),
        "edge_l0": np.ctypeslib.as_array(net.edge_l0, (net.n_edges,)).copy() if net.n_edges else np.zeros(0),
        "edge_wrap": np.ctypeslib.as_array(net.edge_wrap, (net.n_edges,)).astype(np.int8) if net.n_edges else np.zeros(0, np.int8),
        "tri_hjk": np.ctypeslib.as_array(net.tri_hjk, (net.n_triples, 3)).copy() if net.n_triples else np.zeros((0, 3), np.int32),
        "tri_wrap": np.ctypeslib.as_array(net.tri_wrap, (net.n_triples, 2)).astype(np.int8) if net.n_triples else np.zeros((0, 2), np.int8),
    }
    L.or_free_net(C.byref(net))
    return bool(ok), out


def triples_of(points, edge_ij, edge_wrap, offset):
    """or_get_triples on arrays."""
    L = lib()
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 2)
    ij = np.ascontiguousarray(edge_ij, np.int32).reshape(-1, 2)
    w = np.ascontiguousarray(edge_wrap, np.int8)
    net = OrNet()
    net.n_points = len(pts)
    net.n_edges = len(ij)
    net.offset = offset
    keep = (pts, ij, w)
    net.points = _d(pts)
    net.edge_ij = ij.ctypes.data_as(ip)
    net.edge_wrap = w.ctypes.data_as(bp)
    L.or_get_triples(C.byref(net))
    hjk = np.ctypeslib.as_array(net.tri_hjk, (net.n_triples, 3)).copy() if net.n_triples else np.zeros((0, 3), np.int32)
    tw = np.ctypeslib.as_array(net.tri_wrap, (net.n_triples, 2)).astype(np.int8) if net.n_triples else np.zeros((0, 2), np.int8)
    C.CDLL(None).free(net.tri_hjk)
    C.CDLL(None).free(net.tri_wrap)
    del keep
    return hjk, tw


class Model:
    """Holds numpy arrays alive behind an OrModel."""

    def __init__(self, a, ks, kb, fcodes=None):
        self.a = {k: v for k, v in a.items()}
        n = len(a["points"])
        self.edge_ij = np.ascontiguousarray(a["edge_ij"], np.int32)
        self.edge_l0 = np.ascontiguousarray(a["edge_l0"], np.float64)
        self.edge_wrap = np.ascontiguousarray(a["edge_wrap"], np.int8)
        self.tri_hjk = np.ascontiguousarray(a["tri_hjk"], np.int32)
        self.tri_wrap = np.ascontiguousarray(a["tri_wrap"], np.int8)
        if fcodes is None:
            y = a["points"][:, 1]
            fcodes = np.where((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10), 0, 3).astype(np.uint8)
        self.fcodes = np.ascontiguousarray(fcodes, np.uint8)
        self.bond_k = None if a.get("bond_k") is None else np.ascontiguousarray(a["bond_k"], np.float64)
        self.tri_kb = None if a.get("tri_kb") is None else np.ascontiguousarray(a["tri_kb"], np.float64)
        self.tri_phi0 = None if a.get("tri_phi0") is None else np.ascontiguousarray(a["tri_phi0"], np.float64)
        m = OrModel()
        m.n_points = n
        m.n_edges = len(self.edge_l0)
        m.n_triples = len(self.tri_hjk)
        m.width = a["offset"]
        m.ks = ks
        m.kb = kb
        m.edge_ij = self.edge_ij.ctypes.data_as(ip)
        m.edge_l0 = _d(self.edge_l0)
        m.edge_wrap = self.edge_wrap.ctypes.data_as(bp)
        m.tri_hjk = self.tri_hjk.ctypes.data_as(ip)
        m.tri_wrap = self.tri_wrap.ctypes.data_as(bp)
        m.fcodes = self.fcodes.ctypes.data_as(ubp)
        m.bond_k = _d(self.bond_k)
        m.tri_kb = _d(self.tri_kb)
        m.tri_phi0 = _d(self.tri_phi0)
        self.m = m
        self.n = n

    def forces(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        F = np.empty_like(pos)
        lib().or_forces(C.byref(self.m), _d(pos), _d(F))
        return F

    def energies(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        es, eb = C.c_double(), C.c_double()
        lib().or_energies(C.byref(self.m), _d(pos), C.byref(es), C.byref(eb))
        return es.value, eb.value

    def fire(self, pos, params):
        """Relaxes pos (copied); returns (pos, vel, forces, OrReport)."""
        x = np.ascontiguousarray(pos, np.float64).copy()
        v = np.empty_like(x)
        F = np.empty_like(x)
        rep = OrReport()
        lib().or_fire(C.byref(self.m), _d(x), _d(v), _d(F), C.byref(params), C.byref(rep))
        return x, v, F, rep

    def sweep(self, pos, miny, yrange, params, compr, shear, max_records=1000, keep_positions=True):
        x = np.ascontiguousarray(pos, np.float64).copy()
        recs = np.zeros((max_records, 8))
        shp = np.zeros((max_records, self.n, 2)) if keep_positions else None
        c = np.ascontiguousarray(compr, np.float64)
        s = np.ascontiguousarray(shear, np.float64)
        nrec = lib().or_sweep(C.byref(self.m), _d(x), miny, yrange, C.byref(params), _d(c), _d(s), _d(recs),
                              max_records, _d(shp))
        return recs[:nrec], (shp[:nrec] if shp is not None else None), x


def params(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10, max_steps=10**7,
           criterion="max"):
    crit = {"rms": 0, "max": 1}[criterion] if isinstance(criterion, str) else int(criterion)
    return OrParams(alpha0, falpha, dt_max, finc, fdec, nmin, mass, fcut, max_steps, crit)


def affine_displace(pos, miny, yrange, xdisp, ydisp):
    x = np.ascontiguousarray(pos, np.float64).copy()
    lib().or_affine_displace(len(x), _d(x), miny, yrange, xdisp, ydisp)
    return x


def atan2(y, x):
    return lib().or_atan2(float(y), float(x))


def _edges(a):
    ij = np.ascontiguousarray(a["edge_ij"], np.int32).reshape(-1, 2)
    w = np.ascontiguousarray(a["edge_wrap"], np.int8)
    return ij, w


def bond_strains(a, pos0, disp):
    """strain_calc.cpp:96-120 on network arrays a (edge_ij, edge_wrap, offset)."""
    ij, w = _edges(a)
    p0 = np.ascontiguousarray(pos0, np.float64)
    u = np.ascontiguousarray(disp, np.float64)
    out = np.empty(len(ij), np.float64)
    lib().or_bond_strains(len(ij), _i(ij), _b(w), float(a["offset"]), _d(p0), _d(u), _d(out))
    return out


def linear_axial_energy(a, k, pos0, disp):
    """axial_contribution.cpp:64-70, 176-190 (canonical sum)."""
    ij, w = _edges(a)
    p0 = np.ascontiguousarray(pos0, np.float64)
    u = np.ascontiguousarray(disp, np.float64)
    return lib().or_linear_axial_energy(len(ij), _i(ij), _b(w), float(a["offset"]), float(k), _d(p0), _d(u))


def nonaffinity(pos0, disp, miny, axial_strain, shear_strain):
    """na_calc.cpp:308-327 (canonical sum)."""
    p0 = np.ascontiguousarray(pos0, np.float64)
    u = np.ascontiguousarray(disp, np.float64)
    return lib().or_nonaffinity(len(p0), _d(p0), _d(u), float(miny), float(axial_strain), float(shear_strain))


def canon_sum(terms):
    t = np.ascontiguousarray(terms, np.float64)
    return lib().or_canon_sum(_d(t), len(t))


def fire_batch(models, positions, prm, n_threads):
    """Relaxes every model (in place on copies) on n_threads host threads."""
    n = len(models)
    ms = (OrModel * n)(*[m.m for m in models])
    xs = [np.ascontiguousarray(p, np.float64).copy() for p in positions]
    ptrs = (dp * n)(*[_d(x) for x in xs])
    prms = (OrParams * n)(*([prm] * n))
    reps = (OrReport * n)()
    lib().or_fire_batch(n, ms, ptrs, prms, reps, int(n_threads))
    return xs, [reps[i] for i in range(n)]


# ---------------------------------------------------------------- reference

_ref = None


def ref_lib():
    """The reference compiled for the host, or None when unavailable."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        L = C.CDLL(REF_SO)
        L.ref_load_network.restype = C.c_void_p
        L.ref_load_network.argtypes = [C.c_char_p, C.c_int]
        L.ref_free_network.argtypes = [C.c_void_p]
        L.ref_network_info.argtypes = [C.c_void_p, ip, ip, ip, dp, dp, dp]
        L.ref_network_arrays.argtypes = [C.c_void_p, dp, ip, dp, bp, ip, bp]
        L.ref_affine_displace.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.ref_run_fire_md.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp, dp, ip,
                                      dp, bp, ip, bp, ubp, dp, C.c_double, C.c_double, C.c_int, C.c_int, dp, ip]
        L.ref_do_relaxation_run.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_double, C.c_double,
                                            dp, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp]
        L.ref_parse_batch_file.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int, dp, dp, dp, ip, dp,
                                           dp, ip, dp, dp]
        L.ref_lsrelax_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        _ref = L
    return _ref


def ref_read_network(path, want_triples=True):
    L = ref_lib()
    h = L.ref_load_network(str(path).encode(), int(want_triples))
    n, e, t = C.c_int(), C.c_int(), C.c_int()
    off, mny, mxy = C.c_double(), C.c_double(), C.c_double()
    ok = L.ref_network_info(h, C.byref(n), C.byref(e), C.byref(t), C.byref(off), C.byref(mny), C.byref(mxy))
    a = {"points": np.zeros((n.value, 2)), "edge_ij": np.zeros((e.value, 2), np.int32),
         "edge_l0": np.zeros(e.value), "edge_wrap": np.zeros(e.value, np.int8),
         "tri_hjk": np.zeros((t.value, 3), np.int32), "tri_wrap": np.zeros((t.value, 2), np.int8)}
    L.ref_network_arrays(h, _d(a["points"]), a["edge_ij"].ctypes.data_as(ip), _d(a["edge_l0"]),
                         a["edge_wrap"].ctypes.data_as(bp), a["tri_hjk"].ctypes.data_as(ip),
                         a["tri_wrap"].ctypes.data_as(bp))
    L.ref_free_network(h)
    a.update(offset=off.value, miny=mny.value, maxy=mxy.value)
    return bool(ok), a


def ref_run_fire_md(a, pos, ks, kb, fcodes, fire_params, mass, fcut, max_steps, nmin):
    """The reference's run_fire_md (host-compiled) -> (pos, report[3], steps)."""
    L = ref_lib()
    x = np.ascontiguousarray(pos, np.float64).copy()
    v = np.zeros_like(x)
    F = np.zeros_like(x)
    rep = (C.c_double * 3)()
    steps = C.c_int()
    fp = np.ascontiguousarray(fire_params, np.float64)
    ij = np.ascontiguousarray(a["edge_ij"], np.int32)
    l0 = np.ascontiguousarray(a["edge_l0"], np.float64)
    w = np.ascontiguousarray(a["edge_wrap"], np.int8)
    hjk = np.ascontiguousarray(a["tri_hjk"], np.int32)
    tw = np.ascontiguousarray(a["tri_wrap"], np.int8)
    fc = np.ascontiguousarray(fcodes, np.uint8)
    L.ref_run_fire_md(len(x), len(l0), len(hjk), a["offset"], ks, kb, _d(x), _d(v), _d(F), ij.ctypes.data_as(ip),
                      _d(l0), w.ctypes.data_as(bp), hjk.ctypes.data_as(ip), tw.ctypes.data_as(bp),
                      fc.ctypes.data_as(ubp), _d(fp), mass, fcut, max_steps, nmin, rep, C.byref(steps))
    return x, [rep[0], rep[1], rep[2]], steps.value


def ref_affine_displace(pos, miny, yrange, xdisp, ydisp):
    x = np.ascontiguousarray(pos, np.float64).copy()
    ref_lib().ref_affine_displace(len(x), _d(x), miny, yrange, xdisp, ydisp)
    return x
