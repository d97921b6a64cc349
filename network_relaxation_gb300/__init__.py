"""GB300-native FIRE strain-and-relax of 2D elastic fiber networks.

Python face of libnetrelax.so (include/netrelax.h).  Names follow the
reference program (jmichelstl/network_relaxation, src/large_strain_relax.cu):
read_network, get_triples, affine_displace, run_fire_md, do_relaxation_run,
relaxation_batch, parse_batch_file; plus device-resident Network / Batch
objects for repeated relaxations.

Arrays are numpy: positions float64 (N, 2); bonds int32 (E, 2) + l0 float64
(E,) + wrap int8 (E,); triples int32 (T, 3) + wrap int8 (T, 2).
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import (NR_CRIT_MAX, NR_CRIT_RMS, NR_ERR_CAPACITY, NR_ERR_CUDA, NR_ERR_INVALID, NR_ERR_IO,  # noqa: F401
                    NR_ERR_NONFINITE, NR_ERR_OOM, NR_ERR_PARSE, NR_ERR_TIMEOUT, NR_FP64, NR_MIXED,
                    NR_NOT_CONVERGED, NR_OK, BatchSpec, FireParams, MeshBatchSpec, MeshInfo, NetRelaxError, Report,
                    SprInfo, SprRecord, SprSpec, StepRecord, check)

__all__ = [
    "HostNetwork", "Network", "Batch", "fire_params", "read_network", "get_triples", "run_fire_md",
    "parse_batch_file", "do_relaxation_run", "relaxation_batch", "lsrelax_main", "get_file_lists", "lib",
    "NetRelaxError", "FireParams", "Report", "get_strains", "linear_axial_energy", "calc_na_val",
]


def lib():
    """The loaded native library (raises if it is not built)."""
    return _capi.load()


def _dp(a):
    return a.ctypes.data_as(_capi.c_double_p) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_capi.c_int_p) if a is not None else None


def _bp(a):
    return a.ctypes.data_as(_capi.c_schar_p) if a is not None else None


def _stream(stream):
    """Accepts None, an int handle, or a torch.cuda.Stream."""
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def fire_params(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10,
                max_steps=10_000_000, criterion="max", precision="fp64"):
    """FIRE parameters (fire_params[5], nmin, mass, fcut, nmax of the batch
    file; defaults are Bitzek et al. 2006 with a 1e-10 max-force stop)."""
    crit = {"rms": NR_CRIT_RMS, "max": NR_CRIT_MAX}[criterion] if isinstance(criterion, str) else int(criterion)
    prec = {"fp64": NR_FP64, "mixed": NR_MIXED}[precision] if isinstance(precision, str) else int(precision)
    return FireParams(alpha0, falpha, dt_max, finc, fdec, nmin, mass, fcut, max_steps, crit, prec)


class HostNetwork:
    """Topology + positions on the host (nr_host_network)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _capi.load().nr_host_network_free(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @classmethod
    def read(cls, path, strict=True):
        """read_network (large_strain_relax.cu:42).  strict=False returns the
        partially read network on a parse error, as the reference does."""
        out = C.c_void_p()
        st = _capi.load().nr_read_network(str(path).encode(), C.byref(out))
        if st != NR_OK and (strict or not out.value):
            if out.value:
                _capi.load().nr_host_network_free(out)
            raise NetRelaxError(st, "read_network(%s)" % path)
        return cls(out)

    @classmethod
    def read_bin(cls, path):
        """A network saved by write_bin (nr_read_network_bin): no parsing, no
        get_triples; a truncated or corrupt file raises NR_ERR_PARSE."""
        out = C.c_void_p()
        st = _capi.load().nr_read_network_bin(str(path).encode(), C.byref(out))
        if st != NR_OK:
            if out.value:
                _capi.load().nr_host_network_free(out)
            raise NetRelaxError(st, "read_network_bin(%s)" % path)
        return cls(out)

    @classmethod
    def from_arrays(cls, points, edge_ij, edge_wrap, offset, edge_l0=None):
        points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2)
        edge_ij = np.ascontiguousarray(edge_ij, dtype=np.int32).reshape(-1, 2)
        edge_wrap = np.ascontiguousarray(edge_wrap, dtype=np.int8).reshape(-1)
        l0 = None if edge_l0 is None else np.ascontiguousarray(edge_l0, dtype=np.float64)
        out = C.c_void_p()
        check(_capi.load().nr_host_network_from_arrays(len(points), _dp(points), len(edge_ij), _ip(edge_ij), _dp(l0),
                                                       _bp(edge_wrap), float(offset), C.byref(out)),
              "nr_host_network_from_arrays")
        return cls(out)

    @classmethod
    def lattice(cls, nx, ny, p, jitter=0.0, seed=1, line_triples=False):
        """Diluted triangular lattice (nr_gen_lattice)."""
        out = C.c_void_p()
        check(_capi.load().nr_gen_lattice(int(nx), int(ny), float(p), float(jitter), int(seed), int(bool(line_triples)),
                                          C.byref(out)), "nr_gen_lattice")
        return cls(out)

    @classmethod
    def read_mesh(cls, path, strict=True):
        """read_network_mesh (network_mesh_relax.cu:72): a network with its
        gel triangles, areas and duplicate pairs."""
        out = C.c_void_p()
        st = _capi.load().nr_read_network_mesh(str(path).encode(), C.byref(out))
        if st != NR_OK and (strict or not out.value):
            if out.value:
                _capi.load().nr_host_network_free(out)
            raise NetRelaxError(st, "read_network_mesh(%s)" % path)
        return cls(out)

    @classmethod
    def lattice_mesh(cls, nx, ny, p, jitter=0.0, seed=1):
        """Network embedded in a gel on an nx x ny grid (nr_gen_lattice_mesh)."""
        out = C.c_void_p()
        check(_capi.load().nr_gen_lattice_mesh(int(nx), int(ny), float(p), float(jitter), int(seed), C.byref(out)),
              "nr_gen_lattice_mesh")
        return cls(out)

    def set_mesh(self, facets, areas, mesh_pairs=None):
        """Attaches gel triangles and areas; mesh_pairs None finds the
        duplicate pairs as the reader does."""
        f = np.ascontiguousarray(facets, dtype=np.int32).reshape(-1, 3)
        a = np.ascontiguousarray(areas, dtype=np.float64)
        mp = None if mesh_pairs is None else np.ascontiguousarray(mesh_pairs, dtype=np.int32).reshape(-1, 2)
        check(_capi.load().nr_host_network_set_mesh(self._h, len(f), _ip(f), _dp(a), -1 if mp is None else len(mp),
                                                    _ip(mp)), "set_mesh")
        return self

    def set_offset(self, offset):
        check(_capi.load().nr_host_network_set_offset(self._h, float(offset)), "set_offset")
        return self

    def mesh_info(self):
        info = _capi.MeshInfo()
        _capi.load().nr_host_network_mesh_info(self._h, C.byref(info))
        return info

    def reorder(self, method="morton"):
        """Renumbers the nodes for locality (nr_host_network_reorder);
        returns new_to_old (the old index of each new node)."""
        m = {"morton": _capi.NR_ORDER_MORTON, "rcm": _capi.NR_ORDER_RCM}[method]
        perm = np.empty(self.n_points, np.int32)
        check(_capi.load().nr_host_network_reorder(self._h, m, _ip(perm)), "nr_host_network_reorder")
        return perm

    def write_mesh(self, path):
        check(_capi.load().nr_write_network_mesh(self._h, str(path).encode()), "nr_write_network_mesh")

    @classmethod
    def mikado(cls, n_fibers, fiber_len=0.05, k0=1.0, kappa0=1e-5, seed=3):
        out = C.c_void_p()
        check(_capi.load().nr_gen_mikado(int(n_fibers), float(fiber_len), float(k0), float(kappa0), int(seed),
                                         C.byref(out)), "nr_gen_mikado")
        return cls(out)

    def dsm_layout_check(self):
        """Builds the cluster kernels' sub-block layout (item slots, resolved
        incidence, gather records) on the host and checks it
        (nr_dsm_layout_check): a dict of sub-block size, sub-blocks, nodes,
        violations."""
        st = (C.c_longlong * 4)()
        check(_capi.load().nr_dsm_layout_check(self.handle, st), "nr_dsm_layout_check")
        return dict(zip(("sub_block_nodes", "sub_blocks", "nodes", "violations"), (int(v) for v in st)))

    def tile_layout_check(self, ctas=152, target_nodes=512):
        """Builds the tiled kernel's spatial layout on the host and checks
        its invariants (nr_tile_layout_check): a dict of tiles, positions,
        largest tile, largest record (bytes), halo nodes, violations."""
        st = (C.c_longlong * 6)()
        check(_capi.load().nr_tile_layout_check(self.handle, int(ctas), int(target_nodes), st),
              "nr_tile_layout_check")
        keys = ("tiles", "positions", "max_tile_nodes", "max_record_bytes", "halo_nodes", "violations")
        return dict(zip(keys, (int(v) for v in st)))

    def get_triples(self):
        """get_triples (large_strain_relax.cu:116) into this network."""
        check(_capi.load().nr_get_triples(self._h), "get_triples")
        return self

    def set_triples(self, hjk, wrap, kb=None, phi0=None):
        hjk = np.ascontiguousarray(hjk, dtype=np.int32).reshape(-1, 3)
        wrap = np.ascontiguousarray(wrap, dtype=np.int8).reshape(-1, 2)
        kb = None if kb is None else np.ascontiguousarray(kb, dtype=np.float64)
        phi0 = None if phi0 is None else np.ascontiguousarray(phi0, dtype=np.float64)
        check(_capi.load().nr_host_network_set_triples(self._h, len(hjk), _ip(hjk), _bp(wrap), _dp(kb), _dp(phi0)),
              "set_triples")
        return self

    def set_bond_k(self, k):
        k = None if k is None else np.ascontiguousarray(k, dtype=np.float64)
        check(_capi.load().nr_host_network_set_bond_k(self._h, _dp(k)), "set_bond_k")
        return self

    def info(self):
        info = _capi.HostInfo()
        _capi.load().nr_host_network_info(self._h, C.byref(info))
        return info

    @property
    def n_points(self):
        return self.info().n_points

    def arrays(self):
        """dict of numpy copies: points, edge_ij, edge_l0, edge_wrap, tri_hjk,
        tri_wrap and (when set) bond_k, tri_kb, tri_phi0; plus offset, miny,
        maxy."""
        i = self.info()
        a = {
            "points": np.empty((i.n_points, 2), np.float64),
            "edge_ij": np.empty((i.n_edges, 2), np.int32),
            "edge_l0": np.empty(i.n_edges, np.float64),
            "edge_wrap": np.empty(i.n_edges, np.int8),
            "tri_hjk": np.empty((i.n_triples, 3), np.int32),
            "tri_wrap": np.empty((i.n_triples, 2), np.int8),
            "bond_k": np.empty(i.n_edges, np.float64) if i.has_bond_k else None,
            "tri_kb": np.empty(i.n_triples, np.float64) if i.has_tri_kb else None,
            "tri_phi0": np.empty(i.n_triples, np.float64) if i.has_tri_phi0 else None,
        }
        _capi.load().nr_host_network_arrays(self._h, _dp(a["points"]), _ip(a["edge_ij"]), _dp(a["edge_l0"]),
                                            _bp(a["edge_wrap"]), _ip(a["tri_hjk"]), _bp(a["tri_wrap"]),
                                            _dp(a["bond_k"]), _dp(a["tri_kb"]), _dp(a["tri_phi0"]))
        a.update(offset=i.offset, miny=i.miny, maxy=i.maxy)
        m = self.mesh_info()
        a["facets"] = np.empty((m.n_facets, 3), np.int32)
        a["areas"] = np.empty(m.n_areas, np.float64)
        a["mpairs"] = np.empty((m.n_mesh_pairs, 2), np.int32)
        _capi.load().nr_host_network_mesh_arrays(self._h, _ip(a["facets"]), _dp(a["areas"]), _ip(a["mpairs"]))
        a.update(minx=m.minx, maxx=m.maxx)
        return a

    def fcodes(self):
        out = np.empty(self.n_points, np.uint8)
        _capi.load().nr_host_network_fcodes(self._h, out.ctypes.data_as(_capi.c_uchar_p))
        return out

    def write(self, path):
        check(_capi.load().nr_write_network(self._h, str(path).encode()), "nr_write_network")

    def write_bin(self, path):
        """Binary side-car of this network (nr_write_network_bin): arrays as
        stored, triples and mesh included, FNV-1a checksum."""
        check(_capi.load().nr_write_network_bin(self._h, str(path).encode()), "nr_write_network_bin")


def read_network(path):
    """read_network (large_strain_relax.cu:42-114) with the reference's
    outputs: (ok, offset, points[2N], edges[(i, j, l0, wrap)], min_y, max_y)."""
    out = C.c_void_p()
    st = _capi.load().nr_read_network(str(path).encode(), C.byref(out))
    if not out.value:
        return False, 0.0, np.zeros(0), [], 0.0, 0.0
    net = HostNetwork(out)
    a = net.arrays()
    edges = [(int(i), int(j), float(l0), int(w)) for (i, j), l0, w in zip(a["edge_ij"], a["edge_l0"], a["edge_wrap"])]
    return st == NR_OK, a["offset"], a["points"].reshape(-1), edges, a["miny"], a["maxy"]


def get_triples(points, edges, offset):
    """get_triples (large_strain_relax.cu:116-184): list of
    (hinge, j, k, wrap_j, wrap_k)."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 2)
    ij = np.array([(e[0], e[1]) for e in edges], dtype=np.int32).reshape(-1, 2)
    l0 = np.array([e[2] for e in edges], dtype=np.float64)
    w = np.array([e[3] for e in edges], dtype=np.int8)
    net = HostNetwork.from_arrays(pts, ij, w, offset, l0).get_triples()
    a = net.arrays()
    return [(int(h), int(j), int(k), int(wj), int(wk)) for (h, j, k), (wj, wk) in zip(a["tri_hjk"], a["tri_wrap"])]


class Network:
    """A network resident on the GPU (nr_network)."""

    def __init__(self, host, ks=1.0, kb=0.0, stream=None):
        self._lib = _capi.load()
        out = C.c_void_p()
        check(self._lib.nr_network_create(host.handle, float(ks), float(kb), _stream(stream), C.byref(out)),
              "nr_network_create")
        self._h = out
        self.n = self._lib.nr_network_n_points(out)
        info = host.info()
        self.miny, self.maxy = info.miny, info.maxy
        m = host.mesh_info()
        self.minx, self.maxx = m.minx, m.maxx

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.nr_network_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def positions(self, stream=None):
        out = np.empty((self.n, 2), np.float64)
        check(self._lib.nr_network_get_positions(self._h, _dp(out), _stream(stream)), "get_positions")
        return out

    def set_positions(self, xy, stream=None):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(self.n, 2)
        check(self._lib.nr_network_set_positions(self._h, _dp(xy), _stream(stream)), "set_positions")

    def positions_device_ptr(self):
        return self._lib.nr_network_positions_device(self._h)

    def affine_displace(self, miny, yrange, xdisp, ydisp, stream=None):
        check(self._lib.nr_affine_displace(self._h, float(miny), float(yrange), float(xdisp), float(ydisp),
                                           _stream(stream)), "affine_displace")

    def relax(self, params=None, stream=None):
        params = params or fire_params()
        rep = Report()
        st = self._lib.nr_relax(self._h, C.byref(params), C.byref(rep), _stream(stream))
        check(st, "nr_relax")
        return rep

    def forces(self, stream=None):
        out = np.empty((self.n, 2), np.float64)
        check(self._lib.nr_forces(self._h, _dp(out), _stream(stream)), "nr_forces")
        return out

    def energies(self, stream=None):
        es, eb = C.c_double(), C.c_double()
        check(self._lib.nr_energies(self._h, C.byref(es), C.byref(eb), _stream(stream)), "nr_energies")
        return es.value, eb.value

    def plan(self, precision="fp64"):
        """The launch plan the library picks for this network (nr_network_plan)."""
        buf = C.create_string_buffer(256)
        check(self._lib.nr_network_plan(self._h, {"fp64": NR_FP64, "mixed": NR_MIXED}[precision], buf, 256),
              "nr_network_plan")
        return buf.value.decode()

    def stress(self, stream=None):
        """(stress {xx, yy, xy}, energies {E_stretch, E_bend}) at the current
        positions: the virial of the stretch and bending forces over the
        network's area (nr_stress)."""
        st = (C.c_double * 3)()
        en = (C.c_double * 2)()
        check(self._lib.nr_stress(self._h, st, en, _stream(stream)), "nr_stress")
        return np.array(st[:]), (en[0], en[1])

    # ---- gel coupling (network_mesh_relax.cu) ----

    def set_gel(self, smod, bmod, dilation):
        check(self._lib.nr_network_set_gel(self._h, float(smod), float(bmod), float(dilation)), "nr_network_set_gel")

    def gel_inv_mats(self, stream=None):
        check(self._lib.nr_network_gel_inv_mats(self._h, _stream(stream)), "nr_network_gel_inv_mats")

    def dilate(self, minx, miny, factor, stream=None):
        check(self._lib.nr_dilate(self._h, float(minx), float(miny), float(factor), _stream(stream)), "nr_dilate")

    def mesh_energies(self, stream=None):
        """(E_stretch, E_bend, E_gel)."""
        e = (C.c_double * 3)()
        check(self._lib.nr_mesh_energies(self._h, e, _stream(stream)), "nr_mesh_energies")
        return e[0], e[1], e[2]

    def mesh_prepare(self, smod, bmod, dilation, area, stream=None):
        """Dilate, then set the gel with the preferred dilation (returned)."""
        pref = C.c_double()
        check(self._lib.nr_mesh_prepare(self._h, float(smod), float(bmod), float(dilation), float(area),
                                        C.byref(pref), _stream(stream)), "nr_mesh_prepare")
        return pref.value

    def mesh_sweep(self, compr, shear, height, params=None, miny=None, keep_positions=False, max_records=100000,
                   stream=None):
        """network_mesh_relax.cu's compression then shear protocol.  Returns
        (records, shear_positions or None)."""
        return self._sweep(self._lib.nr_mesh_sweep, "nr_mesh_sweep", compr, shear, params, miny, height,
                           keep_positions, max_records, stream)

    def _sweep(self, fn, name, compr, shear, params, miny, yrange, keep_positions, max_records, stream):
        params = params or fire_params()
        miny = self.miny if miny is None else miny
        yrange = (self.maxy - self.miny) if yrange is None else yrange
        c = np.ascontiguousarray(compr, dtype=np.float64)
        s = np.ascontiguousarray(shear, dtype=np.float64)
        n_est = 0
        for r in (c, s):
            if r[1] > 0:
                n_est += 1 + (int((r[1] - r[0]) / r[2] + 1e-9) + 1 if r[2] > 0 else 1)
        n_est = min(max(n_est, 1), max_records)
        recs = (StepRecord * n_est)()
        nrec = C.c_int()
        pos = np.empty((n_est, self.n, 2), np.float64) if keep_positions else None
        st = fn(self._h, float(miny), float(yrange), C.byref(params), _dp(c), _dp(s), recs, n_est, C.byref(nrec),
                _dp(pos), _stream(stream))
        check(st, name)
        recs = [recs[i] for i in range(nrec.value)]
        return recs, (pos[:nrec.value] if pos is not None else None)

    def sweep(self, compr, shear, params=None, miny=None, yrange=None, keep_positions=False, max_records=100000,
              stream=None, graph=False):
        """The compression-then-shear protocol of do_relaxation_run.  Returns
        (records, shear_positions or None).  graph=True runs the whole
        protocol as one CUDA graph (nr_sweep_graph)."""
        fn, name = (self._lib.nr_sweep_graph, "nr_sweep_graph") if graph else (self._lib.nr_sweep, "nr_sweep")
        return self._sweep(fn, name, compr, shear, params, miny, yrange, keep_positions, max_records, stream)


class Batch:
    """Many independent networks relaxed in one launch (nr_batch)."""

    def __init__(self, hosts, ks, kb, stream=None):
        self._lib = _capi.load()
        n = len(hosts)
        handles = (C.c_void_p * n)(*[h.handle.value for h in hosts])
        ks = np.broadcast_to(np.asarray(ks, np.float64), (n,)).copy()
        kb = np.broadcast_to(np.asarray(kb, np.float64), (n,)).copy()
        out = C.c_void_p()
        check(self._lib.nr_batch_create(n, handles, _dp(ks), _dp(kb), _stream(stream), C.byref(out)),
              "nr_batch_create")
        self._h = out
        self.n = n
        self.sizes = np.array([h.n_points for h in hosts])
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        infos = [h.info() for h in hosts]
        self.miny = np.array([i.miny for i in infos])
        self.maxy = np.array([i.maxy for i in infos])

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.nr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def positions(self, stream=None):
        out = np.empty((int(self.offsets[-1]), 2), np.float64)
        check(self._lib.nr_batch_get_positions(self._h, _dp(out), _stream(stream)), "batch get_positions")
        return out

    def set_positions(self, xy, stream=None):
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        check(self._lib.nr_batch_set_positions(self._h, _dp(xy), _stream(stream)), "batch set_positions")

    def positions_device_ptr(self):
        return self._lib.nr_batch_positions_device(self._h)

    def affine_displace(self, xdisp, ydisp, miny=None, yrange=None, stream=None):
        n = self.n
        miny = self.miny if miny is None else np.broadcast_to(np.asarray(miny, np.float64), (n,))
        yrange = (self.maxy - self.miny) if yrange is None else np.broadcast_to(np.asarray(yrange, np.float64), (n,))
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (n,))) for a in
                (miny, yrange, xdisp, ydisp)]
        check(self._lib.nr_batch_affine_displace(self._h, *[_dp(a) for a in arrs], _stream(stream)),
              "batch affine_displace")

    def relax(self, params=None, stream=None):
        params = params or fire_params()
        reps = (Report * self.n)()
        st = self._lib.nr_batch_relax(self._h, C.byref(params), reps, _stream(stream))
        check(st, "nr_batch_relax")
        return [reps[i] for i in range(self.n)]

    def plan(self, precision="mixed"):
        """The launch plan of nr_batch_relax for this batch (nr_batch_plan)."""
        buf = C.create_string_buffer(256)
        check(self._lib.nr_batch_plan(self._h, {"fp64": NR_FP64, "mixed": NR_MIXED}[precision], buf, 256),
              "nr_batch_plan")
        return buf.value.decode()

    def sweep(self, compr, shear, params=None, graph=True, max_steps=100000, stream=None):
        """The strain protocol on every network at once (nr_batch_sweep);
        returns records[step][network].  graph=True records the whole
        protocol as one CUDA graph."""
        params = params or fire_params()
        c = (C.c_double * 3)(*[float(v) for v in compr])
        s = (C.c_double * 3)(*[float(v) for v in shear])
        recs = (StepRecord * (max_steps * self.n))()
        ns = C.c_int()
        st = self._lib.nr_batch_sweep(self._h, C.byref(params), c, s, recs, int(max_steps), C.byref(ns), int(bool(graph)),
                                      _stream(stream))
        check(st, "nr_batch_sweep")
        k = min(ns.value, max_steps)
        return [[recs[j * self.n + i] for i in range(self.n)] for j in range(k)]


def _analysis_arrays(pos0, disp, edges):
    p0 = np.ascontiguousarray(pos0, np.float64).reshape(-1, 2)
    u = np.ascontiguousarray(disp, np.float64).reshape(-1, 2)
    if u.shape != p0.shape:
        raise ValueError("point and displacement count mismatch")
    ij = w = None
    if edges is not None:
        ij = np.ascontiguousarray(edges[0], np.int32).reshape(-1, 2)
        w = np.ascontiguousarray(edges[1], np.int8).reshape(-1)
    return p0, u, ij, w


def get_strains(points, edges, offset, disps, stream=None):
    """get_strains (strain_calc.cpp:96-120) on the GPU: per-bond
    (l_final - l_initial) / l_initial.  edges = (ij[E, 2], wrap[E])."""
    p0, u, ij, w = _analysis_arrays(points, disps, edges)
    out = np.empty(len(ij), np.float64)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(_capi.load().nr_bond_strains(len(p0), len(ij), float(offset), vp(p0), vp(u), vp(ij), vp(w), vp(out),
                                       _stream(stream)), "nr_bond_strains")
    return out


def linear_axial_energy(points, edges, offset, disps, k, stream=None):
    """axial_contribution.cpp:64-70, 176-190 on the GPU: k/2 sum over bonds of
    the squared projection of the relative displacement on the bond."""
    p0, u, ij, w = _analysis_arrays(points, disps, edges)
    e = C.c_double()
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(_capi.load().nr_linear_axial_energy(len(p0), len(ij), float(offset), float(k), vp(p0), vp(u), vp(ij),
                                              vp(w), C.byref(e), _stream(stream)), "nr_linear_axial_energy")
    return e.value


def calc_na_val(points, disps, miny, axial_strain, shear_strain, stream=None):
    """calc_na_val (na_calc.cpp:308-327) on the GPU: mean square deviation of
    the displacement field from the affine one."""
    p0, u, _, _ = _analysis_arrays(points, disps, None)
    na = C.c_double()
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(_capi.load().nr_nonaffinity(len(p0), vp(p0), vp(u), float(miny), float(axial_strain), float(shear_strain),
                                      C.byref(na), _stream(stream)), "nr_nonaffinity")
    return na.value


def run_fire_md(num_dof, npairs, ntriples, width, ks, kb, d_pos, d_vel, d_forces, d_pair_list, d_lengths,
                d_e_offsets, d_triples, d_t_offsets, d_fcodes, fire_params_, mass, fcut, max_steps, nmin, stream=None):
    """run_fire_md (large_strain_relax.cu:596) on device pointers (ints, e.g.
    torch tensor data_ptr()).  Returns (status, report_data[3], step_count)."""
    fp = (C.c_double * 5)(*[float(v) for v in fire_params_])
    rep = (C.c_double * 3)()
    steps = C.c_int()
    vp = lambda p: C.c_void_p(int(p)) if p else None  # noqa: E731
    st = _capi.load().nr_run_fire_md(int(num_dof), int(npairs), int(ntriples), float(width), float(ks), float(kb),
                                     vp(d_pos), vp(d_vel), vp(d_forces), vp(d_pair_list), vp(d_lengths),
                                     vp(d_e_offsets), vp(d_triples), vp(d_t_offsets), vp(d_fcodes), fp, float(mass),
                                     float(fcut), int(max_steps), int(nmin), rep, C.byref(steps), _stream(stream))
    check(st, "run_fire_md")
    return st, [rep[0], rep[1], rep[2]], steps.value


def mesh_run_fire_md(num_dof, npairs, ntriples, nelems, width, ks, kb, smod, bmod, dilation, d_pos, d_vel, d_forces,
                     d_pair_list, d_lengths, d_e_offsets, d_triples, d_t_offsets, d_elems, d_areas, d_inv_mats,
                     d_mpairs, n_mpairs, d_fcodes, fire_params_, mass, fcut, max_steps, nmin, stream=None):
    """run_fire_md (network_mesh_relax.cu:865) on device pointers.  Returns
    (status, report_data[4], step_count)."""
    fp = (C.c_double * 5)(*[float(v) for v in fire_params_])
    rep = (C.c_double * 4)()
    steps = C.c_int()
    vp = lambda p: C.c_void_p(int(p)) if p else None  # noqa: E731
    st = _capi.load().nr_mesh_run_fire_md(
        int(num_dof), int(npairs), int(ntriples), int(nelems), float(width), float(ks), float(kb), float(smod),
        float(bmod), float(dilation), vp(d_pos), vp(d_vel), vp(d_forces), vp(d_pair_list), vp(d_lengths),
        vp(d_e_offsets), vp(d_triples), vp(d_t_offsets), vp(d_elems), vp(d_areas), vp(d_inv_mats), vp(d_mpairs),
        int(n_mpairs), vp(d_fcodes), fp, float(mass), float(fcut), int(max_steps), int(nmin), rep, C.byref(steps),
        _stream(stream))
    check(st, "mesh_run_fire_md")
    return st, [rep[i] for i in range(4)], steps.value


def get_inv_mats(n_facets, d_pos, d_facets, d_inv_mats, stream=None):
    """get_inv_mats (network_mesh_relax.cu:503) on device pointers."""
    vp = lambda p: C.c_void_p(int(p)) if p else None  # noqa: E731
    check(_capi.load().nr_get_inv_mats(int(n_facets), vp(d_pos), vp(d_facets), vp(d_inv_mats), _stream(stream)),
          "get_inv_mats")


def parse_batch_file(path):
    """parse_batch_file (large_strain_relax.cu:297): a BatchSpec."""
    spec = BatchSpec()
    check(_capi.load().nr_parse_batch_file(str(path).encode(), C.byref(spec)), "parse_batch_file", ok=(NR_OK,))
    return spec


def get_file_lists(base, ext="dat", tag=""):
    """get_file_lists (file_lists.cpp:80): list of (dat, log, disp, edata)."""
    lib_ = _capi.load()
    n = lib_.nr_get_file_lists(str(base).encode(), ext.encode(), tag.encode(), None, 0)
    if n < 0:
        raise NetRelaxError(n, "get_file_lists")
    cap = 1 << 16
    while True:
        buf = C.create_string_buffer(cap)
        n = lib_.nr_get_file_lists(str(base).encode(), ext.encode(), tag.encode(), buf, cap)
        if n != NR_ERR_CAPACITY:
            break
        cap *= 4
    if n < 0:
        raise NetRelaxError(n, "get_file_lists")
    parts = buf.raw.split(b"\0")[: 4 * n]
    return [tuple(p.decode() for p in parts[4 * i: 4 * i + 4]) for i in range(n)]


def do_relaxation_run(net_file, log_name, edata_name, disp_base, spec, precision="fp64", criterion="rms"):
    """do_relaxation_run (large_strain_relax.cu:792) with a BatchSpec."""
    prec = {"fp64": NR_FP64, "mixed": NR_MIXED}[precision]
    crit = {"rms": NR_CRIT_RMS, "max": NR_CRIT_MAX}[criterion]
    return check(_capi.load().nr_do_relaxation_run(str(net_file).encode(), str(log_name).encode(),
                                                   str(edata_name).encode(), str(disp_base).encode(), C.byref(spec),
                                                   prec, crit), "do_relaxation_run")


def relaxation_batch(batch_file, precision="fp64", criterion="rms"):
    """relaxation_batch (large_strain_relax.cu:1016)."""
    prec = {"fp64": NR_FP64, "mixed": NR_MIXED}[precision]
    crit = {"rms": NR_CRIT_RMS, "max": NR_CRIT_MAX}[criterion]
    return check(_capi.load().nr_relaxation_batch(str(batch_file).encode(), prec, crit), "relaxation_batch")


def lsrelax_main(argv):
    """The lsrelax command line (large_strain_relax.cu:1047)."""
    args = ["lsrelax"] + list(argv)
    arr = (C.c_char_p * len(args))(*[a.encode() for a in args])
    return _capi.load().nr_lsrelax_main(len(args), arr)


def parse_mesh_batch_file(path):
    """parse_batch_file (network_mesh_relax.cu:413): a MeshBatchSpec."""
    spec = MeshBatchSpec()
    check(_capi.load().nr_parse_mesh_batch_file(str(path).encode(), C.byref(spec)), "parse_mesh_batch_file",
          ok=(NR_OK,))
    return spec


def do_mesh_relaxation_run(net_file, log_name, edata_name, disp_base, spec, criterion="rms"):
    """do_relaxation_run (network_mesh_relax.cu:1095) with a MeshBatchSpec."""
    crit = {"rms": NR_CRIT_RMS, "max": NR_CRIT_MAX}[criterion]
    return check(_capi.load().nr_do_mesh_relaxation_run(str(net_file).encode(), str(log_name).encode(),
                                                        str(edata_name).encode(), str(disp_base).encode(),
                                                        C.byref(spec), crit), "do_mesh_relaxation_run")


def mesh_relaxation_batch(batch_file, criterion="rms"):
    """relaxation_batch (network_mesh_relax.cu:1393)."""
    crit = {"rms": NR_CRIT_RMS, "max": NR_CRIT_MAX}[criterion]
    return check(_capi.load().nr_mesh_relaxation_batch(str(batch_file).encode(), crit), "mesh_relaxation_batch")


def nmrelax_main(argv):
    """The nmrelax command line (network_mesh_relax.cu:1424)."""
    args = ["nmrelax"] + list(argv)
    arr = (C.c_char_p * len(args))(*[a.encode() for a in args])
    return _capi.load().nr_nmrelax_main(len(args), arr)


# ------------------------------------------------------------ linear response

def spr_assemble(host, ks, kb, mu):
    """get_sparse_stiffness_mat (sparse_relax.cpp:434): upper-triangle
    (rows, cols, vals) in (row, col) order.  Host only."""
    lib_ = _capi.load()
    n = lib_.nr_spr_assemble(host.handle, float(ks), float(kb), float(mu), None, None, None)
    if n < 0:
        raise NetRelaxError(int(n), "nr_spr_assemble")
    rows, cols, vals = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
    lib_.nr_spr_assemble(host.handle, float(ks), float(kb), float(mu), rows.ctypes.data_as(C.POINTER(C.c_long)),
                         cols.ctypes.data_as(C.POINTER(C.c_long)), _dp(vals))
    return rows, cols, vals


class Spr:
    """The linear-response problem of sparse_relax.cpp on the GPU (nr_spr)."""

    def __init__(self, host, ks=1.0, kb=0.0, mu=0.0, stream=None):
        self._lib = _capi.load()
        out = C.c_void_p()
        check(self._lib.nr_spr_create(host.handle, float(ks), float(kb), float(mu), _stream(stream), C.byref(out)),
              "nr_spr_create")
        self._h = out
        self.n = host.n_points

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.nr_spr_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def info(self):
        i = SprInfo()
        self._lib.nr_spr_info(self._h, C.byref(i))
        return i

    def solve(self, affine=True, tol=1e-12, max_iter=None, stream=None):
        """The unit compression and shear loads (NR_OK or NR_NOT_CONVERGED)."""
        if max_iter is None:
            max_iter = max(1000, min(10 * self.info().n_free_dofs, 10_000_000))
        return check(self._lib.nr_spr_solve(self._h, int(bool(affine)), float(tol), int(max_iter), _stream(stream)),
                     "nr_spr_solve")

    def point(self, compression, shear, want_u=True, stream=None):
        """(SprRecord, full displacement field (N, 2) or None)."""
        rec = SprRecord()
        u = np.empty((self.n, 2), np.float64) if want_u else None
        check(self._lib.nr_spr_point(self._h, float(compression), float(shear), C.byref(rec), _dp(u),
                                     _stream(stream)), "nr_spr_point")
        return rec, u


def parse_spr_batch_file(path):
    """parse_batch_file (sparse_relax.cpp:931): an SprSpec."""
    spec = SprSpec()
    check(_capi.load().nr_parse_spr_batch_file(str(path).encode(), C.byref(spec)), "parse_spr_batch_file",
          ok=(NR_OK,))
    return spec


def spr_do_relaxation_run(dat_name, log_name, disp_base, e_name, spec, strain_mode=False, affine=True, itemize=False):
    """do_relaxation_run (sparse_relax.cpp:676)."""
    return check(_capi.load().nr_spr_do_relaxation_run(str(dat_name).encode(), str(log_name).encode(),
                                                       str(disp_base).encode(), str(e_name).encode(), C.byref(spec),
                                                       int(strain_mode), int(affine), int(itemize)),
                 "spr_do_relaxation_run")


def sp_relax_main(argv):
    """The sp_relax command line (sparse_relax.cpp:1165)."""
    args = ["sp_relax"] + list(argv)
    arr = (C.c_char_p * len(args))(*[a.encode() for a in args])
    return _capi.load().nr_sp_relax_main(len(args), arr)
