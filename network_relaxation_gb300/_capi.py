"""ctypes bindings of include/netrelax.h (libnetrelax.so, built in-tree).

Loading fails loudly when the library is missing: there is no Python or CPU
fallback for anything that runs on the GPU.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnetrelax.so")

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_schar_p = C.POINTER(C.c_byte)
c_uchar_p = C.POINTER(C.c_ubyte)

NR_OK = 0
NR_NOT_CONVERGED = 1
NR_ERR_INVALID = -1
NR_ERR_IO = -2
NR_ERR_PARSE = -3
NR_ERR_CUDA = -4
NR_ERR_OOM = -5
NR_ERR_NONFINITE = -6
NR_ERR_TIMEOUT = -7
NR_ERR_CAPACITY = -8
NR_CRIT_RMS = 0
NR_CRIT_MAX = 1
NR_FP64 = 0
NR_MIXED = 1
NR_ORDER_MORTON = 1
NR_ORDER_RCM = 2


class HostInfo(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_edges", C.c_int), ("n_triples", C.c_int), ("offset", C.c_double),
                ("miny", C.c_double), ("maxy", C.c_double), ("has_bond_k", C.c_int), ("has_tri_kb", C.c_int),
                ("has_tri_phi0", C.c_int)]


class FireParams(C.Structure):
    _fields_ = [("alpha0", C.c_double), ("falpha", C.c_double), ("dt_max", C.c_double), ("finc", C.c_double),
                ("fdec", C.c_double), ("nmin", C.c_int), ("mass", C.c_double), ("fcut", C.c_double),
                ("max_steps", C.c_int), ("criterion", C.c_int), ("precision", C.c_int)]


class Report(C.Structure):
    _fields_ = [("rms_force", C.c_double), ("e_stretch", C.c_double), ("e_bend", C.c_double),
                ("max_force", C.c_double), ("steps", C.c_int), ("status", C.c_int), ("fp64_steps", C.c_int),
                ("reserved", C.c_int), ("e_gel", C.c_double), ("stress_xx", C.c_double), ("stress_yy", C.c_double),
                ("stress_xy", C.c_double)]


class StepRecord(C.Structure):
    _fields_ = [("curr_disp", C.c_double), ("max_comp", C.c_double), ("e_stretch", C.c_double),
                ("e_bend", C.c_double), ("rms_force", C.c_double), ("max_force", C.c_double), ("steps", C.c_int),
                ("is_shear", C.c_int), ("status", C.c_int), ("fp64_steps", C.c_int), ("e_gel", C.c_double),
                ("stress_xx", C.c_double), ("stress_yy", C.c_double), ("stress_xy", C.c_double)]


class SprInfo(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_free_dofs", C.c_int), ("n_triples", C.c_int), ("nnz_upper", C.c_long),
                ("sell_entries", C.c_long), ("iterations", C.c_int * 2), ("rel_residual", C.c_double * 2),
                ("minx", C.c_double), ("maxx", C.c_double), ("miny", C.c_double), ("maxy", C.c_double)]


class SprRecord(C.Structure):
    _fields_ = [("compression", C.c_double), ("shear", C.c_double), ("e_total", C.c_double), ("e_ss", C.c_double),
                ("e_bend", C.c_double), ("residual", C.c_double), ("iterations", C.c_int), ("status", C.c_int)]


class SprSpec(C.Structure):
    _fields_ = [("base", C.c_char * 1024), ("tag", C.c_char * 256), ("ks", C.c_double), ("kb", C.c_double),
                ("mu", C.c_double), ("compr", C.c_double * 3), ("shear", C.c_double * 3)]


class MeshInfo(C.Structure):
    _fields_ = [("n_facets", C.c_int), ("n_areas", C.c_int), ("n_mesh_pairs", C.c_int), ("minx", C.c_double),
                ("maxx", C.c_double)]


class BatchSpec(C.Structure):
    _fields_ = [("base", C.c_char * 1024), ("tag", C.c_char * 256), ("ks", C.c_double), ("kb", C.c_double),
                ("fire_params", C.c_double * 5), ("nmin", C.c_int), ("mass", C.c_double), ("fcut", C.c_double),
                ("nmax", C.c_int), ("compr", C.c_double * 3), ("shear", C.c_double * 3), ("absolute", C.c_int),
                ("stress_columns", C.c_int)]


class MeshBatchSpec(C.Structure):
    _fields_ = [("net", BatchSpec), ("bmod", C.c_double), ("smod", C.c_double), ("dilation", C.c_double)]


P = C.c_void_p
# name -> (restype, argtypes)
SIGNATURES = {
    "nr_status_string": (C.c_char_p, [C.c_int]),
    "nr_last_error": (C.c_char_p, []),
    "nr_abi_version": (C.c_int, []),
    "nr_read_network": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "nr_get_triples": (C.c_int, [P]),
    "nr_host_network_from_arrays": (C.c_int, [C.c_int, c_double_p, C.c_int, c_int_p, c_double_p, c_schar_p,
                                              C.c_double, C.POINTER(P)]),
    "nr_host_network_set_triples": (C.c_int, [P, C.c_int, c_int_p, c_schar_p, c_double_p, c_double_p]),
    "nr_host_network_set_bond_k": (C.c_int, [P, c_double_p]),
    "nr_host_network_info": (None, [P, C.POINTER(HostInfo)]),
    "nr_host_network_arrays": (None, [P, c_double_p, c_int_p, c_double_p, c_schar_p, c_int_p, c_schar_p, c_double_p,
                                      c_double_p, c_double_p]),
    "nr_host_network_fcodes": (None, [P, c_uchar_p]),
    "nr_write_network": (C.c_int, [P, C.c_char_p]),
    "nr_write_network_bin": (C.c_int, [P, C.c_char_p]),
    "nr_read_network_bin": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "nr_write_positions": (C.c_int, [c_double_p, C.c_int, C.c_char_p]),
    "nr_host_network_free": (None, [P]),
    "nr_host_network_reorder": (C.c_int, [P, C.c_int, c_int_p]),
    "nr_gen_lattice": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_int, C.POINTER(P)]),
    "nr_gen_mikado": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, C.POINTER(P)]),
    "nr_network_create": (C.c_int, [P, C.c_double, C.c_double, P, C.POINTER(P)]),
    "nr_network_destroy": (C.c_int, [P]),
    "nr_network_n_points": (C.c_int, [P]),
    "nr_network_set_positions": (C.c_int, [P, c_double_p, P]),
    "nr_network_get_positions": (C.c_int, [P, c_double_p, P]),
    "nr_network_positions_device": (C.c_void_p, [P]),
    "nr_affine_displace": (C.c_int, [P, C.c_double, C.c_double, C.c_double, C.c_double, P]),
    "nr_relax": (C.c_int, [P, C.POINTER(FireParams), C.POINTER(Report), P]),
    "nr_forces": (C.c_int, [P, c_double_p, P]),
    "nr_energies": (C.c_int, [P, c_double_p, c_double_p, P]),
    "nr_stress": (C.c_int, [P, c_double_p, c_double_p, P]),
    "nr_batch_sweep": (C.c_int, [P, C.POINTER(FireParams), c_double_p, c_double_p, C.POINTER(StepRecord), C.c_int,
                                 c_int_p, C.c_int, P]),
    "nr_tuning_load": (C.c_int, [C.c_char_p]),
    "nr_tuning_value": (C.c_double, [C.c_char_p]),
    "nr_tuning_source": (C.c_char_p, []),
    "nr_network_plan": (C.c_int, [P, C.c_int, C.c_char_p, C.c_size_t]),
    "nr_tile_layout_check": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_longlong)]),
    "nr_dsm_layout_check": (C.c_int, [P, C.POINTER(C.c_longlong)]),
    "nr_batch_plan": (C.c_int, [P, C.c_int, C.c_char_p, C.c_size_t]),
    "nr_sweep": (C.c_int, [P, C.c_double, C.c_double, C.POINTER(FireParams), c_double_p, c_double_p,
                           C.POINTER(StepRecord), C.c_int, c_int_p, c_double_p, P]),
    "nr_sweep_graph": (C.c_int, [P, C.c_double, C.c_double, C.POINTER(FireParams), c_double_p, c_double_p,
                                 C.POINTER(StepRecord), C.c_int, c_int_p, c_double_p, P]),
    "nr_run_fire_md": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, P, P, P, P, P, P, P,
                                 P, P, c_double_p, C.c_double, C.c_double, C.c_int, C.c_int, c_double_p, c_int_p, P]),
    "nr_read_network_mesh": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "nr_write_network_mesh": (C.c_int, [P, C.c_char_p]),
    "nr_host_network_set_mesh": (C.c_int, [P, C.c_int, c_int_p, c_double_p, C.c_int, c_int_p]),
    "nr_host_network_set_offset": (C.c_int, [P, C.c_double]),
    "nr_host_network_mesh_info": (None, [P, C.POINTER(MeshInfo)]),
    "nr_host_network_mesh_arrays": (None, [P, c_int_p, c_double_p, c_int_p]),
    "nr_gen_lattice_mesh": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, C.POINTER(P)]),
    "nr_network_set_gel": (C.c_int, [P, C.c_double, C.c_double, C.c_double]),
    "nr_network_gel_inv_mats": (C.c_int, [P, P]),
    "nr_dilate": (C.c_int, [P, C.c_double, C.c_double, C.c_double, P]),
    "nr_mesh_energies": (C.c_int, [P, c_double_p, P]),
    "nr_mesh_prepare": (C.c_int, [P, C.c_double, C.c_double, C.c_double, C.c_double, c_double_p, P]),
    "nr_mesh_sweep": (C.c_int, [P, C.c_double, C.c_double, C.POINTER(FireParams), c_double_p, c_double_p,
                                C.POINTER(StepRecord), C.c_int, c_int_p, c_double_p, P]),
    "nr_get_inv_mats": (C.c_int, [C.c_int, P, P, P, P]),
    "nr_mesh_run_fire_md": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_double, P, P, P, P, P, P, P, P, P, P, P, P,
                                      C.c_int, P, c_double_p, C.c_double, C.c_double, C.c_int, C.c_int, c_double_p,
                                      c_int_p, P]),
    "nr_spr_assemble": (C.c_long, [P, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_long),
                                    C.POINTER(C.c_long), c_double_p]),
    "nr_spr_create": (C.c_int, [P, C.c_double, C.c_double, C.c_double, P, C.POINTER(P)]),
    "nr_spr_destroy": (C.c_int, [P]),
    "nr_spr_info": (None, [P, C.POINTER(SprInfo)]),
    "nr_spr_solve": (C.c_int, [P, C.c_int, C.c_double, C.c_int, P]),
    "nr_spr_point": (C.c_int, [P, C.c_double, C.c_double, C.POINTER(SprRecord), c_double_p, P]),
    "nr_parse_spr_batch_file": (C.c_int, [C.c_char_p, C.POINTER(SprSpec)]),
    "nr_spr_do_relaxation_run": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(SprSpec),
                                           C.c_int, C.c_int, C.c_int]),
    "nr_spr_relaxation_batch": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int]),
    "nr_sp_relax_main": (C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
    "nr_bond_strains": (C.c_int, [C.c_int, C.c_int, C.c_double, P, P, P, P, P, P]),
    "nr_linear_axial_energy": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, P, P, P, P, c_double_p, P]),
    "nr_nonaffinity": (C.c_int, [C.c_int, P, P, C.c_double, C.c_double, C.c_double, c_double_p, P]),
    "nr_energies_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, P, P, P, P, P,
                                      P, P, P]),
    "nr_batch_create": (C.c_int, [C.c_int, C.POINTER(P), c_double_p, c_double_p, P, C.POINTER(P)]),
    "nr_batch_destroy": (C.c_int, [P]),
    "nr_batch_size": (C.c_int, [P]),
    "nr_batch_last_launches": (C.c_int, [P]),
    "nr_batch_total_points": (C.c_int, [P]),
    "nr_batch_set_positions": (C.c_int, [P, c_double_p, P]),
    "nr_batch_get_positions": (C.c_int, [P, c_double_p, P]),
    "nr_batch_positions_device": (C.c_void_p, [P]),
    "nr_batch_affine_displace": (C.c_int, [P, c_double_p, c_double_p, c_double_p, c_double_p, P]),
    "nr_batch_relax": (C.c_int, [P, C.POINTER(FireParams), C.POINTER(Report), P]),
    "nr_parse_batch_file": (C.c_int, [C.c_char_p, C.POINTER(BatchSpec)]),
    "nr_get_file_lists": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t]),
    "nr_do_relaxation_run": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(BatchSpec),
                                       C.c_int, C.c_int]),
    "nr_relaxation_batch": (C.c_int, [C.c_char_p, C.c_int, C.c_int]),
    "nr_lsrelax_main": (C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
    "nr_parse_mesh_batch_file": (C.c_int, [C.c_char_p, C.POINTER(MeshBatchSpec)]),
    "nr_do_mesh_relaxation_run": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                            C.POINTER(MeshBatchSpec), C.c_int]),
    "nr_mesh_relaxation_batch": (C.c_int, [C.c_char_p, C.c_int]),
    "nr_nmrelax_main": (C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
}

_lib = None


def load():
    """Loads libnetrelax.so (raises OSError with a build hint when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError("libnetrelax.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"` "
                      "or `python network_relaxation_gb300/build.py`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class NetRelaxError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.nr_last_error().decode(errors="replace")
        name = lib.nr_status_string(status).decode()
        super().__init__("%s failed: %s (%d)%s" % (where, name, status, (": " + msg) if msg else ""))
        self.status = status


def check(status, where, ok=(NR_OK, NR_NOT_CONVERGED)):
    if status not in ok:
        raise NetRelaxError(status, where)
    return status
