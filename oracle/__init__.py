"""Python bindings of the oracle (nr_oracle.c, nr_oracle_mesh.c) and of the
reference compiled for the host (oracle/_ref/liblsr_ref.so and
oracle/_ref/libnmr_ref.so, present only where the reference checkout exists).

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
REF_MESH_SO = os.path.join(HERE, "_ref", "libnmr_ref.so")
REF_SPR_SO = os.path.join(HERE, "_ref", "libspr_ref.so")
REF_NA_SO = os.path.join(HERE, "_ref", "libna_ref.so")
SOURCES = ["nr_oracle.c", "nr_oracle_mesh.c", "nr_oracle_spr.c", "nr_oracle.h", "nr_oracle_internal.h"]
lp = C.POINTER(C.c_long)

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
                ("tri_phi0", dp), ("n_elems", C.c_int), ("n_mpairs", C.c_int), ("smod", C.c_double),
                ("bmod", C.c_double), ("gel_dilation", C.c_double), ("elems", ip), ("inv_mats", dp),
                ("areas", dp), ("mpairs", ip)]


class OrParams(C.Structure):
    _fields_ = [("alpha0", C.c_double), ("falpha", C.c_double), ("dt_max", C.c_double), ("finc", C.c_double),
                ("fdec", C.c_double), ("nmin", C.c_int), ("mass", C.c_double), ("fcut", C.c_double),
                ("max_steps", C.c_int), ("criterion", C.c_int)]


class OrReport(C.Structure):
    _fields_ = [("rms_force", C.c_double), ("max_force", C.c_double), ("e_stretch", C.c_double),
                ("e_bend", C.c_double), ("steps", C.c_int), ("converged", C.c_int), ("e_gel", C.c_double)]


class OrMesh(C.Structure):
    _fields_ = [("net", OrNet), ("n_facets", C.c_int), ("n_areas", C.c_int), ("n_mpairs", C.c_int), ("facets", ip),
                ("areas", dp),
                ("mpairs", ip), ("minx", C.c_double), ("maxx", C.c_double)]


def build(force=False):
    """Compiles libnr_oracle.so (gcc, seconds)."""
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in SOURCES):
        subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True)
    return ORACLE_SO


_ref_built = False


def build_ref():
    """Builds oracle/_ref/liblsr_ref.so (and libnmr_ref.so) when the reference
    checkout exists; once per process."""
    global _ref_built
    if not _ref_built:
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)
        _ref_built = True
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
        L.or_virial.argtypes = [C.POINTER(OrModel), dp, dp]
        L.or_virial.restype = None
        L.or_fire.argtypes = [C.POINTER(OrModel), dp, dp, dp, C.POINTER(OrParams), C.POINTER(OrReport)]
        L.or_sweep.restype = C.c_int
        L.or_sweep.argtypes = [C.POINTER(OrModel), dp, C.c_double, C.c_double, C.POINTER(OrParams), dp, dp, dp,
                               C.c_int, dp]
        L.or_fire_batch.argtypes = [C.c_int, C.POINTER(OrModel), C.POINTER(dp), C.POINTER(OrParams),
                                    C.POINTER(OrReport), C.c_int]
        L.or_read_network_mesh.argtypes = [C.c_char_p, C.POINTER(OrMesh)]
        L.or_free_mesh.argtypes = [C.POINTER(OrMesh)]
        L.or_mesh_pairs.restype = C.c_int
        L.or_mesh_pairs.argtypes = [C.c_int, dp, C.c_double, C.c_double, ip]
        L.or_inv_mats.argtypes = [C.c_int, dp, ip, dp]
        L.or_dilate.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double]
        L.or_gel_forces.argtypes = [C.POINTER(OrModel), dp, dp]
        L.or_gel_energy.restype = C.c_double
        L.or_gel_energy.argtypes = [C.POINTER(OrModel), dp]
        L.or_preferred_dilation.restype = C.c_double
        L.or_preferred_dilation.argtypes = [C.c_double] * 5
        L.or_spr_stiffness.restype = C.c_long
        L.or_spr_stiffness.argtypes = [C.c_int, dp, C.c_int, ip, dp, bp, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, ip, bp, lp, lp, dp]
        L.or_spr_energies.argtypes = [dp, C.c_int, ip, dp, bp, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_int, ip, bp, dp, dp, dp]
        L.or_spr_bc.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, ubp, dp]
        L.or_mesh_sweep.restype = C.c_int
        L.or_mesh_sweep.argtypes = [C.POINTER(OrModel), dp, C.c_double, C.c_double, C.POINTER(OrParams), dp, dp,
                                    dp, C.c_int, dp]
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


def _splitmix64(seed, count):
    """The first `count` outputs of SplitMix64 (Steele, Lea & Flood, OOPSLA
    2014) from `seed`, as uint64: output k mixes seed + (k + 1) * golden."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (np.arange(1, count + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def gen_lattice(nx, ny, p, seed, jitter=0.0):
    """Restatement of the library's diluted triangular lattice (the
    synthetic inputs of the benchmarks; the reference ships none): nx x ny
    nodes, unit spacing, rows at y = j sqrt(3)/2, odd rows shifted by +0.5,
    x-periodic with period nx.  SplitMix64 draws, in order: with jitter > 0
    two per node (dx, dy in U(-jitter, jitter); rows 0 and ny-1 move in x
    only), then per node in row-major order three, one for each of its right,
    up-left and up-right bonds, kept when the draw is below p.  Rest lengths
    as read_network computes them (large_strain_relax.cu:97-99).  No
    triples (use triples_of).  Returns the dict read_network returns."""
    n = nx * ny
    row = np.sqrt(3.0) / 2.0
    jj, ii = np.divmod(np.arange(n), nx)
    pts = np.empty((n, 2))
    pts[:, 0] = ii + 0.5 * (jj & 1)
    pts[:, 1] = jj * row
    k0 = 0
    if jitter > 0:
        u = (_splitmix64(seed, 2 * n) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        dx = jitter * (2.0 * u[0::2] - 1.0)
        dy = jitter * (2.0 * u[1::2] - 1.0)
        pts[:, 0] += dx
        inner = (jj != 0) & (jj != ny - 1)
        pts[inner, 1] += dy[inner]
        k0 = 2 * n
    u = (_splitmix64(seed, k0 + 3 * n)[k0:] >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    u = u.reshape(n, 3)
    odd = (jj & 1) == 1
    cand = []  # (node order, slot, i, j, wrap)
    right = (jj * nx + (ii + 1) % nx, np.where(ii == nx - 1, 1, 0))
    up_l_i = np.where(odd, ii, ii - 1)
    up_l = ((jj + 1) * nx + np.where(up_l_i < 0, up_l_i + nx, up_l_i), np.where(up_l_i < 0, -1, 0))
    up_r_i = np.where(odd, ii + 1, ii)
    up_r = ((jj + 1) * nx + np.where(up_r_i >= nx, up_r_i - nx, up_r_i), np.where(up_r_i >= nx, 1, 0))
    has_up = jj + 1 < ny
    keep = np.stack([u[:, 0] < p, has_up & (u[:, 1] < p), has_up & (u[:, 2] < p)], axis=1)
    other = np.stack([right[0], up_l[0], up_r[0]], axis=1)
    wrap = np.stack([right[1], up_l[1], up_r[1]], axis=1)
    src = np.repeat(np.arange(n)[:, None], 3, axis=1)
    ij = np.stack([src[keep], other[keep]], axis=1).astype(np.int32)
    w = wrap[keep].astype(np.int8)
    dxb = pts[ij[:, 1], 0] + nx * w.astype(np.float64) - pts[ij[:, 0], 0]
    dyb = pts[ij[:, 1], 1] - pts[ij[:, 0], 1]
    l0 = np.sqrt(dxb * dxb + dyb * dyb)
    y = pts[:, 1]
    miny = min(float(np.finfo(np.float32).max), float(y.min()))
    maxy = max(float(np.finfo(np.float32).tiny), float(y.max()))
    return {"offset": float(nx), "miny": miny, "maxy": maxy, "points": pts, "edge_ij": ij, "edge_l0": l0,
            "edge_wrap": w, "tri_hjk": np.zeros((0, 3), np.int32), "tri_wrap": np.zeros((0, 2), np.int8)}


def lattice_with_triples(nx, ny, p, seed):
    """gen_lattice plus get_triples (large_strain_relax.cu:116-184)."""
    a = gen_lattice(nx, ny, p, seed)
    a["tri_hjk"], a["tri_wrap"] = triples_of(a["points"], a["edge_ij"], a["edge_wrap"], a["offset"])
    return a


class Model:
    """Holds numpy arrays alive behind an OrModel."""

    def __init__(self, a, ks, kb, fcodes=None, gel=None):
        """gel: None or dict(elems (F,3), inv_mats (F,6), areas (F,), mpairs
        (P,2), smod, bmod, dilation) -- the network_mesh_relax.cu model."""
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
        if gel is not None:
            self.elems = np.ascontiguousarray(gel["elems"], np.int32).reshape(-1, 3)
            self.inv_mats = np.ascontiguousarray(gel["inv_mats"], np.float64).reshape(-1, 6)
            self.areas = np.ascontiguousarray(gel["areas"], np.float64)
            self.mpairs = np.ascontiguousarray(gel["mpairs"], np.int32).reshape(-1, 2)
            m.n_elems = len(self.elems)
            m.n_mpairs = len(self.mpairs)
            m.smod = gel["smod"]
            m.bmod = gel["bmod"]
            m.gel_dilation = gel["dilation"]
            m.elems = _i(self.elems)
            m.inv_mats = _d(self.inv_mats)
            m.areas = _d(self.areas)
            m.mpairs = _i(self.mpairs)
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

    def virial(self, pos):
        """{W_xx, W_yy, W_xy} of the stretch and bending forces at pos
        (or_virial); the stress is W / area."""
        pos = np.ascontiguousarray(pos, np.float64)
        w = np.zeros(3)
        lib().or_virial(C.byref(self.m), _d(pos), _d(w))
        return w

    def fire(self, pos, params):
        """Relaxes pos (copied); returns (pos, vel, forces, OrReport)."""
        x = np.ascontiguousarray(pos, np.float64).copy()
        v = np.empty_like(x)
        F = np.empty_like(x)
        rep = OrReport()
        lib().or_fire(C.byref(self.m), _d(x), _d(v), _d(F), C.byref(params), C.byref(rep))
        return x, v, F, rep

    def gel_energy(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        return lib().or_gel_energy(C.byref(self.m), _d(pos))

    def mesh_sweep(self, pos, miny, height, params, compr, shear, max_records=1000, keep_positions=True):
        """network_mesh_relax.cu's compression then shear protocol on a
        prepared (dilated) model; records of 9 values."""
        x = np.ascontiguousarray(pos, np.float64).copy()
        recs = np.zeros((max_records, 9))
        shp = np.zeros((max_records, self.n, 2)) if keep_positions else None
        c = np.ascontiguousarray(compr, np.float64)
        s = np.ascontiguousarray(shear, np.float64)
        nrec = lib().or_mesh_sweep(C.byref(self.m), _d(x), miny, height, C.byref(params), _d(c), _d(s), _d(recs),
                                   max_records, _d(shp))
        return recs[:nrec], (shp[:nrec] if shp is not None else None), x

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


_ref_na = None


def ref_nonaffinity(pos0, disp, minx, miny, axial_strain, shear_strain):
    """The reference's own calc_na_val (na_calc.cpp:308-327, a sequential
    sum), built for the host by build_ref.sh; None where it is not built."""
    global _ref_na
    if _ref_na is None:
        if not os.path.exists(REF_NA_SO):
            return None
        _ref_na = C.CDLL(REF_NA_SO)
        _ref_na.ref_calc_na_val.restype = C.c_double
        _ref_na.ref_calc_na_val.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.c_double, C.c_double]
    p0 = np.ascontiguousarray(pos0, np.float64)
    u = np.ascontiguousarray(disp, np.float64)
    return _ref_na.ref_calc_na_val(len(p0), _d(p0), _d(u), float(minx), float(miny), float(axial_strain),
                                   float(shear_strain))


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


# ------------------------------------------------------------ mesh composites

def read_network_mesh(path, triple_offset=None):
    """or_read_network_mesh -> (ok, dict); triples from or_get_triples with
    period triple_offset (default: the file's offset)."""
    L = lib()
    mesh = OrMesh()
    ok = L.or_read_network_mesh(str(path).encode(), C.byref(mesh))
    net = mesh.net

    def arr(ptr, shape, dtype):
        n = int(np.prod(shape))
        return np.ctypeslib.as_array(ptr, shape).astype(dtype) if n and ptr else np.zeros(shape, dtype)

    a = {
        "offset": net.offset, "miny": net.miny, "maxy": net.maxy, "minx": mesh.minx, "maxx": mesh.maxx,
        "points": arr(net.points, (net.n_points, 2), np.float64),
        "edge_ij": arr(net.edge_ij, (net.n_edges, 2), np.int32),
        "edge_l0": arr(net.edge_l0, (net.n_edges,), np.float64),
        "edge_wrap": arr(net.edge_wrap, (net.n_edges,), np.int8),
        "facets": arr(mesh.facets, (mesh.n_facets, 3), np.int32),
        "areas": arr(mesh.areas, (mesh.n_areas,), np.float64),
        "mpairs": arr(mesh.mpairs, (mesh.n_mpairs, 2), np.int32),
    }
    L.or_free_mesh(C.byref(mesh))
    if len(a["points"]):
        a["tri_hjk"], a["tri_wrap"] = triples_of(a["points"], a["edge_ij"], a["edge_wrap"],
                                                 a["offset"] if triple_offset is None else triple_offset)
    else:
        a["tri_hjk"], a["tri_wrap"] = np.zeros((0, 3), np.int32), np.zeros((0, 2), np.int8)
    return bool(ok), a


def mesh_pairs(points, offset, minx):
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 2)
    out = np.zeros((max(1, len(pts)), 2), np.int32)
    n = lib().or_mesh_pairs(len(pts), _d(pts), float(offset), float(minx), _i(out))
    return out[:n].copy()


def inv_mats(pos, elems):
    p = np.ascontiguousarray(pos, np.float64)
    el = np.ascontiguousarray(elems, np.int32).reshape(-1, 3)
    out = np.zeros((len(el), 6))
    lib().or_inv_mats(len(el), _d(p), _i(el), _d(out))
    return out


def dilate(pos, minx, miny, factor):
    x = np.ascontiguousarray(pos, np.float64).copy()
    lib().or_dilate(len(x), _d(x), float(minx), float(miny), float(factor))
    return x


def preferred_dilation(ks, e_stretch_dilated, area, dilation, bmod):
    return lib().or_preferred_dilation(float(ks), float(e_stretch_dilated), float(area), float(dilation), float(bmod))


def mesh_gel(a, smod, bmod, dilation, inv=None):
    """The gel dict Model takes, inverse matrices from a's points."""
    return {"elems": a["facets"], "inv_mats": inv_mats(a["points"], a["facets"]) if inv is None else inv,
            "areas": a["areas"], "mpairs": a["mpairs"], "smod": smod, "bmod": bmod, "dilation": dilation}


# ------------------------------------------------------ linear response (SPR)

def _spr_args(a):
    """Arrays of network a with the triples get_sparse_stiffness_mat computes
    itself (sparse_relax.cpp:444-446: get_triples on the points and bonds)."""
    pts = np.ascontiguousarray(a["points"], np.float64)
    ij = np.ascontiguousarray(a["edge_ij"], np.int32)
    l0 = np.ascontiguousarray(a["edge_l0"], np.float64)
    w = np.ascontiguousarray(a["edge_wrap"], np.int8)
    hjk, tw = triples_of(pts, ij, w, a["offset"]) if len(pts) else (np.zeros((0, 3), np.int32),
                                                                     np.zeros((0, 2), np.int8))
    return pts, ij, l0, w, np.ascontiguousarray(hjk, np.int32), np.ascontiguousarray(tw, np.int8)


def spr_stiffness(a, ks, kb, mu):
    """get_sparse_stiffness_mat (sparse_relax.cpp:434): upper-triangle
    triplets (rows, cols, vals) in (row, col) order."""
    L = lib()
    pts, ij, l0, w, hjk, tw = _spr_args(a)
    args = (len(pts), _d(pts), len(l0), _i(ij), _d(l0), _b(w), float(a["offset"]), float(ks), float(kb), float(mu),
            len(hjk), _i(hjk), _b(tw))
    n = L.or_spr_stiffness(*args, None, None, None)
    rows, cols, vals = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
    L.or_spr_stiffness(*args, rows.ctypes.data_as(lp), cols.ctypes.data_as(lp), _d(vals))
    return rows, cols, vals


def spr_energies(a, ks, kb, mu, u):
    """get_stretch_shear_energy + get_bending_energy (sparse_relax.cpp:49-96)."""
    pts, ij, l0, w, hjk, tw = _spr_args(a)
    uu = np.ascontiguousarray(u, np.float64)
    ess, eb = C.c_double(), C.c_double()
    lib().or_spr_energies(_d(pts), len(l0), _i(ij), _d(l0), _b(w), float(a["offset"]), float(ks), float(kb),
                          float(mu), len(hjk), _i(hjk), _b(tw), _d(uu), C.byref(ess), C.byref(eb))
    return ess.value, eb.value


def spr_protocol(a, ks, kb, mu, compr, shear, strain_mode=True, affine=True, minx=None, maxx=None):
    # (run_relaxation_batch's rule that an increment of a range narrower than
    # 1e-10 becomes 1e12 is the caller's.)
    """do_relaxation_run of sparse_relax.cpp:676-870 restated with numpy on a
    dense matrix (small networks): records of (compression, shear, e_total,
    e_ss, e_bend, residual) and the full displacement fields.  The sparse
    SPQR solve becomes a dense least-squares solve (the same solution for a
    full-rank system)."""
    pts = np.ascontiguousarray(a["points"], np.float64)
    n = len(pts)
    miny, maxy = a["miny"], a["maxy"]
    if minx is None:
        minx, maxx = pts[:, 0].min(), pts[:, 0].max()
    y = pts[:, 1]
    bottom = y < miny + 1e-10
    top = y > maxy - 1e-10
    free = ~(bottom | top)
    (cmin, cmax, cinc), (smin, smax, sinc) = [list(v) for v in (compr, shear)]
    if strain_mode:
        cmin, cmax, cinc = (v * (maxy - miny) for v in (cmin, cmax, cinc))
        smin, smax, sinc = (v * (maxx - minx) for v in (smin, smax, sinc))
    rows, cols, vals = spr_stiffness(a, ks, kb, mu)
    K = np.zeros((2 * n, 2 * n))
    K[rows, cols] = vals
    K[cols, rows] = vals
    dof = np.repeat(free, 2)
    Kff, Kfa = K[np.ix_(dof, dof)], K[dof, :]
    bc = np.zeros(2 * n)
    is_top = top.astype(np.uint8)
    recs, fields = [], []
    c = cmin
    while c < cmax + 1e-10:
        sh = smin
        while sh < smax + 1e-10:
            lib().or_spr_bc(n, _d(pts), miny, maxy, c, sh, int(affine), is_top.ctypes.data_as(ubp), _d(bc))
            rhs = -(Kfa @ bc)
            u = np.linalg.lstsq(Kff, rhs, rcond=None)[0]
            uf = bc.copy()
            uf[dof] += u
            ess, eb = spr_energies(a, ks, kb, mu, uf)
            recs.append((c, sh, ess + eb, ess, eb, float(np.linalg.norm(rhs - Kff @ u))))
            fields.append(uf)
            if not sinc > 0:  # the reference loops forever on a zero increment
                break
            sh += sinc
        if not cinc > 0:
            break
        c += cinc
    return recs, fields


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


_ref_mesh = None


def ref_mesh_lib():
    """network_mesh_relax.cu compiled for the host, or None when unavailable."""
    global _ref_mesh
    if _ref_mesh is None:
        if not os.path.exists(REF_MESH_SO):
            return None
        L = C.CDLL(REF_MESH_SO)
        L.ref_load_mesh.restype = C.c_void_p
        L.ref_load_mesh.argtypes = [C.c_char_p, C.c_int, C.c_double]
        L.ref_free_mesh.argtypes = [C.c_void_p]
        L.ref_mesh_info.argtypes = [C.c_void_p, ip, dp]
        L.ref_mesh_arrays.argtypes = [C.c_void_p, dp, ip, dp, bp, ip, bp, ip, dp, ip]
        L.ref_get_inv_mats.argtypes = [C.c_int, C.c_int, dp, ip, dp]
        L.ref_dilate.argtypes = [C.c_int, dp, C.c_double, C.c_double, C.c_double]
        L.ref_mesh_forces.argtypes = ([C.c_int] * 5 + [C.c_double] * 6 +
                                      [dp, ip, dp, bp, ip, bp, ip, dp, dp, ip, ubp, dp])
        L.ref_gel_energies.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, ip, dp, dp, dp]
        L.ref_mesh_run_fire_md.argtypes = ([C.c_int] * 5 + [C.c_double] * 6 +
                                           [dp, ip, dp, bp, ip, bp, ip, dp, dp, ip, ubp, dp, C.c_double, C.c_double,
                                            C.c_int, C.c_int, dp, ip])
        L.ref_mesh_do_relaxation_run.argtypes = ([C.c_char_p] * 4 + [C.c_double] * 5 +
                                                 [dp, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp])
        L.ref_mesh_parse_batch_file.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int, dp, dp, ip,
                                                dp, dp, ip, dp, dp]
        L.ref_nmrelax_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        _ref_mesh = L
    return _ref_mesh


def ref_read_network_mesh(path, triple_offset=None):
    """The reference's read_network_mesh (+ get_triples with period
    triple_offset, default the file's offset) -> (ok, dict)."""
    L = ref_mesh_lib()
    h = L.ref_load_mesh(str(path).encode(), 1, -1.0 if triple_offset is None else float(triple_offset))
    counts = (C.c_int * 6)()
    box = (C.c_double * 5)()
    ok = L.ref_mesh_info(h, counts, box)
    n, e, t, f, p, na = list(counts)
    a = {"points": np.zeros((n, 2)), "edge_ij": np.zeros((e, 2), np.int32), "edge_l0": np.zeros(e),
         "edge_wrap": np.zeros(e, np.int8), "tri_hjk": np.zeros((t, 3), np.int32), "tri_wrap": np.zeros((t, 2), np.int8),
         "facets": np.zeros((f, 3), np.int32), "areas": np.zeros(na), "mpairs": np.zeros((p, 2), np.int32)}
    L.ref_mesh_arrays(h, _d(a["points"]), _i(a["edge_ij"]), _d(a["edge_l0"]), _b(a["edge_wrap"]), _i(a["tri_hjk"]),
                      _b(a["tri_wrap"]), _i(a["facets"]), _d(a["areas"]), _i(a["mpairs"]))
    L.ref_free_mesh(h)
    a.update(offset=box[0], minx=box[1], miny=box[2], maxx=box[3], maxy=box[4])
    return bool(ok), a


def _ref_model_args(a, gel, fcodes):
    ij = np.ascontiguousarray(a["edge_ij"], np.int32)
    l0 = np.ascontiguousarray(a["edge_l0"], np.float64)
    w = np.ascontiguousarray(a["edge_wrap"], np.int8)
    hjk = np.ascontiguousarray(a["tri_hjk"], np.int32)
    tw = np.ascontiguousarray(a["tri_wrap"], np.int8)
    el = np.ascontiguousarray(gel["elems"], np.int32)
    ar = np.ascontiguousarray(gel["areas"], np.float64)
    inv = np.ascontiguousarray(gel["inv_mats"], np.float64)
    mp = np.ascontiguousarray(gel["mpairs"], np.int32)
    fc = np.ascontiguousarray(fcodes, np.uint8)
    keep = (ij, l0, w, hjk, tw, el, ar, inv, mp, fc)
    counts = [len(l0), len(hjk), len(el), len(mp)]
    ptrs = [_i(ij), _d(l0), _b(w), _i(hjk), _b(tw), _i(el), _d(ar), _d(inv), _i(mp), fc.ctypes.data_as(ubp)]
    return keep, counts, ptrs


def ref_mesh_forces(a, pos, width, ks, kb, gel, fcodes):
    """One force evaluation by the reference's kernels, run_fire_md's order."""
    L = ref_mesh_lib()
    x = np.ascontiguousarray(pos, np.float64)
    F = np.zeros_like(x)
    keep, counts, ptrs = _ref_model_args(a, gel, fcodes)
    L.ref_mesh_forces(len(x), *counts, width, ks, kb, gel["smod"], gel["bmod"], gel["dilation"], _d(x), *ptrs, _d(F))
    del keep
    return F


def ref_gel_energies(pos, gel):
    L = ref_mesh_lib()
    x = np.ascontiguousarray(pos, np.float64)
    el = np.ascontiguousarray(gel["elems"], np.int32)
    ar = np.ascontiguousarray(gel["areas"], np.float64)
    inv = np.ascontiguousarray(gel["inv_mats"], np.float64)
    out = np.zeros(len(el))
    L.ref_gel_energies(len(x), len(el), gel["smod"], gel["bmod"], gel["dilation"], _d(x), _i(el), _d(ar), _d(inv),
                       _d(out))
    return out


def ref_mesh_run_fire_md(a, pos, width, ks, kb, gel, fcodes, fire_params, mass, fcut, max_steps, nmin):
    """network_mesh_relax.cu's run_fire_md (host-compiled) ->
    (pos, report[4], steps)."""
    L = ref_mesh_lib()
    x = np.ascontiguousarray(pos, np.float64).copy()
    keep, counts, ptrs = _ref_model_args(a, gel, fcodes)
    rep = (C.c_double * 4)()
    steps = C.c_int()
    fp = np.ascontiguousarray(fire_params, np.float64)
    L.ref_mesh_run_fire_md(len(x), *counts, width, ks, kb, gel["smod"], gel["bmod"], gel["dilation"], _d(x), *ptrs,
                           _d(fp), mass, fcut, max_steps, nmin, rep, C.byref(steps))
    del keep
    return x, [rep[i] for i in range(4)], steps.value


def ref_dilate(pos, minx, miny, factor):
    x = np.ascontiguousarray(pos, np.float64).copy()
    ref_mesh_lib().ref_dilate(len(x), _d(x), float(minx), float(miny), float(factor))
    return x


def ref_get_inv_mats(pos, elems):
    p = np.ascontiguousarray(pos, np.float64)
    el = np.ascontiguousarray(elems, np.int32).reshape(-1, 3)
    out = np.zeros((len(el), 6))
    ref_mesh_lib().ref_get_inv_mats(len(p), len(el), _d(p), _i(el), _d(out))
    return out


_ref_spr = None


def ref_spr_lib():
    """sparse_relax.cpp compiled for the host (dense CHOLMOD / SPQR
    stand-ins), or None when unavailable."""
    global _ref_spr
    if _ref_spr is None:
        if not os.path.exists(REF_SPR_SO):
            return None
        L = C.CDLL(REF_SPR_SO)
        L.ref_spr_load.restype = C.c_void_p
        L.ref_spr_load.argtypes = [C.c_char_p]
        L.ref_spr_free.argtypes = [C.c_void_p]
        L.ref_spr_info.argtypes = [C.c_void_p, ip, dp]
        L.ref_spr_arrays.argtypes = [C.c_void_p, dp, ip, dp, bp, ip, bp]
        L.ref_spr_stiffness.restype = C.c_long
        L.ref_spr_stiffness.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, lp, lp, dp]
        L.ref_spr_energies.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, dp, dp, dp]
        L.ref_spr_do_relaxation_run.argtypes = [C.c_char_p] * 4 + [C.c_double] * 3 + [dp, dp, C.c_int, C.c_int,
                                                                                        C.c_int]
        L.ref_spr_parse_batch_file.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int, dp, dp, dp]
        L.ref_spr_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        _ref_spr = L
    return _ref_spr


class RefSpr:
    """A network loaded by sparse_relax.cpp's own read_network / get_triples."""

    def __init__(self, path):
        self.L = ref_spr_lib()
        self.h = self.L.ref_spr_load(str(path).encode())
        counts = (C.c_int * 3)()
        box = (C.c_double * 5)()
        self.ok = bool(self.L.ref_spr_info(self.h, counts, box))
        n, e, t = list(counts)
        a = {"points": np.zeros((n, 2)), "edge_ij": np.zeros((e, 2), np.int32), "edge_l0": np.zeros(e),
             "edge_wrap": np.zeros(e, np.int8), "tri_hjk": np.zeros((t, 3), np.int32), "tri_wrap": np.zeros((t, 1), np.int8)}
        self.L.ref_spr_arrays(self.h, _d(a["points"]), _i(a["edge_ij"]), _d(a["edge_l0"]), _b(a["edge_wrap"]),
                              _i(a["tri_hjk"]), _b(a["tri_wrap"]))
        a.update(offset=box[0], minx=box[1], maxx=box[2], miny=box[3], maxy=box[4])
        self.a = a

    def stiffness(self, ks, kb, mu):
        n = self.L.ref_spr_stiffness(self.h, ks, kb, mu, None, None, None)
        rows, cols, vals = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
        self.L.ref_spr_stiffness(self.h, ks, kb, mu, rows.ctypes.data_as(lp), cols.ctypes.data_as(lp), _d(vals))
        return rows, cols, vals

    def energies(self, ks, kb, mu, u):
        uu = np.ascontiguousarray(u, np.float64)
        ess, eb = C.c_double(), C.c_double()
        self.L.ref_spr_energies(self.h, ks, kb, mu, _d(uu), C.byref(ess), C.byref(eb))
        return ess.value, eb.value

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_spr_free(self.h)
            self.h = None
