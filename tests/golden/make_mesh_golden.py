"""Regenerates the gel-coupling fixtures in tests/golden/mesh/ from the
reference's own network_mesh_relax.cu (compiled for the host by
oracle/build_ref.sh into oracle/_ref/libnmr_ref.so).

Run where the reference checkout exists:
    python tests/golden/make_mesh_golden.py

Fixtures (inputs come from this project's seeded generator or are written
below; outputs are the reference's):
  mesh/m1.nmc              12 x 9 network-in-gel composite (p = 0.8,
                           jitter 0.15, seed 5)
  mesh/sweep.nmc           10 x 8 composite (p = 0.85, jitter 0.1, seed 7)
  mesh/edge_cases/*.nmc    reader edge cases
  mesh/ref_readers.json    read_network_mesh's result and arrays per file
                           (floats as hex strings; triples with the file's
                           offset)
  mesh/ref_m1.npz          for m1: get_inv_mats; a perturbed configuration
                           and the forces of run_fire_md's kernel sequence
                           (axial, bending, gel_forces, duplicate_forces) at
                           three (ks, kb); gel_energy per element; and one
                           run_fire_md relaxation from an affine shear start
  mesh/ref_sweep/          do_relaxation_run on sweep.nmc: log (without the
                           elapsed-time line), edata and .pos files
  mesh/ref_batch.json      parse_batch_file's results on mesh/batch_files/
"""
import ctypes as C
import glob
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import network_relaxation_gb300 as nr  # noqa: E402
import oracle  # noqa: E402

MESH = os.path.join(HERE, "mesh")
FIRE = [0.1, 0.99, 0.1, 1.1, 0.5]
GEL = dict(smod=0.7, bmod=2.0, dilation=0.05)
FORCE_CASES = [(0.0, 0.0), (1.0, 0.0), (1.0, 1e-2)]
SWEEP = dict(ks=1.0, kb=1e-3, bmod=0.5, smod=0.3, dilation=0.04, nmin=5, mass=1.0, fcut=1e-9, nmax=100000,
             compr=[0.0, 0.02, 0.01], shear=[0.01, 0.03, 0.01])

SQUARE = "0 0\n1 0\n0 1\n1 1\n"
EDGE_CASES = {
    "ok_square.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "comments_blanks.nmc": "4 2 2 1.0\n\n0 0\n# c\n1 0\n0 1\n\n1 1\n0 1 0\nx\n2 3 0\n0 1 3\n\n0 3 2\n#\n0.5\n0.5\n",
    "bad_header.nmc": "4 2 2\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "negative_offset.nmc": "4 2 2 -1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "too_few_points.nmc": "4 2 2 1.0\n0 0\n1 0\n",
    "oob_edge.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 4 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "too_few_edges.nmc": "4 3 0 1.0\n" + SQUARE + "0 1 0\n2 3 0\n",
    "no_facets.nmc": "4 2 0 1.0\n" + SQUARE + "0 1 0\n2 3 0\n",
    "edges_then_eof.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0",
    "oob_facet.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 4\n0 3 2\n0.5\n0.5\n",
    "too_few_facets.nmc": "4 2 3 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n",
    "facets_then_eof.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2",
    "missing_areas.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n",
    "zero_area.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0\n",
    "too_few_areas.nmc": "4 2 2 1.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n",
    "dup_points.nmc": ("7 2 2 1.0\n0 0\n1 0\n0 1\n1 1\n0 1\n1e-12 0.5\n1 0.5\n"
                       "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n"),
    "zero_offset.nmc": "4 2 2 0.0\n" + SQUARE + "0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "unpaired.nmc": "4 2 2 1.0\n0 0\n1 0.25\n0 1\n1 1\n0 1 0\n2 3 0\n0 1 3\n0 3 2\n0.5\n0.5\n",
    "wrapped_bonds.nmc": ("6 4 2 2.0\n0 0\n1 0\n2 0\n0 1\n1 1\n2 1\n0 1 0\n1 0 1\n3 4 0\n4 3 1\n"
                          "0 1 4\n0 4 3\n0.5\n0.5\n"),
}

BATCH_FILES = {
    "ok.txt": "# gel\nnet tagA\n1.0 0.001 0.5 0.3 0.04\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-9 100000\n0 0.02 0.01\n"
              "0.01 0.03 0.01\n",
    "three_values.txt": "net\n1.0 0.001 0.5\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-9 100000\n0 0 0\n0.01 0.03 0.01\n",
    "two_values.txt": "net\n1.0 0.001\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-9 100000\n0 0 0\n0.01 0.03 0.01\n",
    "negative_bmod.txt": "net\n1.0 0.001 -0.5 0.3 0.04\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-9 100000\n0 0 0\n"
                         "0.01 0.03 0.01\n",
    "bad_range.txt": "net\n1.0 0.001 0.5 0.3 0.04\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-9 100000\n0 0 0\n"
                     "0.1 0.01 0.01\n",
}


def hexes(a):
    return [float(v).hex() for v in np.asarray(a, np.float64).reshape(-1)]


def reader_record(path):
    ok, a = oracle.ref_read_network_mesh(path)
    rec = {"ok": ok}
    for k in ("points", "edge_l0", "areas"):
        rec[k] = hexes(a[k])
    for k in ("edge_ij", "edge_wrap", "tri_hjk", "tri_wrap", "facets", "mpairs"):
        rec[k] = np.asarray(a[k]).astype(int).reshape(-1).tolist()
    for k in ("offset", "minx", "miny", "maxx", "maxy"):
        rec[k] = float(a[k]).hex()
    return rec


def fcodes_of(a):
    y = a["points"][:, 1]
    return np.where((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10), 0, 3).astype(np.uint8)


def main():
    if oracle.build_ref() is None or oracle.ref_mesh_lib() is None:
        sys.exit("the reference checkout is needed to regenerate these fixtures")
    os.makedirs(os.path.join(MESH, "edge_cases"), exist_ok=True)
    os.makedirs(os.path.join(MESH, "batch_files"), exist_ok=True)
    nr.HostNetwork.lattice_mesh(12, 9, 0.8, 0.15, seed=5).write_mesh(os.path.join(MESH, "m1.nmc"))
    nr.HostNetwork.lattice_mesh(10, 8, 0.85, 0.1, seed=7).write_mesh(os.path.join(MESH, "sweep.nmc"))
    for name, text in EDGE_CASES.items():
        with open(os.path.join(MESH, "edge_cases", name), "w") as f:
            f.write(text)
    readers = {"m1.nmc": reader_record(os.path.join(MESH, "m1.nmc"))}
    for name in sorted(EDGE_CASES):
        readers["edge_cases/" + name] = reader_record(os.path.join(MESH, "edge_cases", name))
    with open(os.path.join(MESH, "ref_readers.json"), "w") as f:
        json.dump(readers, f, indent=0, sort_keys=True)

    ok, a = oracle.ref_read_network_mesh(os.path.join(MESH, "m1.nmc"))
    assert ok
    fc = fcodes_of(a)
    inv = oracle.ref_get_inv_mats(a["points"], a["facets"])
    gel = {"elems": a["facets"], "inv_mats": inv, "areas": a["areas"], "mpairs": a["mpairs"], **GEL}
    rng = np.random.default_rng(11)
    x = a["points"] + rng.normal(0.0, 0.03, a["points"].shape) * (fc[:, None] > 0)
    for i, j in a["mpairs"]:
        x[j] = x[i] + [a["offset"], 0.0]
    out = {"inv_mats": inv, "x_pert": x, "fcodes": fc}
    for c, (ks, kb) in enumerate(FORCE_CASES):
        out["forces_%d" % c] = oracle.ref_mesh_forces(a, x, a["offset"], ks, kb, gel, fc)
    out["gel_energies"] = oracle.ref_gel_energies(x, gel)
    H = a["maxy"] - a["miny"]
    x0 = oracle.ref_affine_displace(a["points"], a["miny"], H, 0.05 * H, 0.0)
    xr, rep, steps = oracle.ref_mesh_run_fire_md(a, x0, a["offset"], 1.0, 1e-2, gel, fc, FIRE, 1.0, 1e-9, 200000, 5)
    out.update(x_affine=x0, fire_pos=xr, fire_report=np.array(rep), fire_steps=np.array(steps))
    np.savez_compressed(os.path.join(MESH, "ref_m1.npz"), **out)

    sweep_dir = os.path.join(MESH, "ref_sweep")
    shutil.rmtree(sweep_dir, ignore_errors=True)
    os.makedirs(sweep_dir)
    S = SWEEP
    dbl = lambda v: (C.c_double * len(v))(*v)  # noqa: E731
    oracle.ref_mesh_lib().ref_mesh_do_relaxation_run(
        os.path.join(MESH, "sweep.nmc").encode(), os.path.join(sweep_dir, "sweep_log.txt").encode(),
        os.path.join(sweep_dir, "sweep_edata.txt").encode(), os.path.join(sweep_dir, "sweep").encode(), S["ks"],
        S["kb"], S["bmod"], S["smod"], S["dilation"], dbl(FIRE), S["nmin"], S["mass"], S["fcut"], S["nmax"],
        dbl(S["compr"]), dbl(S["shear"]))
    log = os.path.join(sweep_dir, "sweep_log.txt")
    lines = [ln for ln in open(log) if not ln.startswith("Elapsed time")]
    with open(log, "w") as f:
        f.writelines(lines)
    with open(os.path.join(sweep_dir, "params.json"), "w") as f:
        json.dump({"fire": FIRE, **S}, f, indent=1)

    batch = {}
    for name, text in BATCH_FILES.items():
        path = os.path.join(MESH, "batch_files", name)
        with open(path, "w") as f:
            f.write(text)
        base, tag = C.create_string_buffer(1024), C.create_string_buffer(256)
        mech, fp = (C.c_double * 5)(), (C.c_double * 5)()
        nmin, nmax = C.c_int(), C.c_int()
        mass, fcut = C.c_double(), C.c_double()
        compr, shear = (C.c_double * 3)(), (C.c_double * 3)()
        ok = oracle.ref_mesh_lib().ref_mesh_parse_batch_file(path.encode(), base, 1024, tag, 256, mech, fp,
                                                             C.byref(nmin), C.byref(mass), C.byref(fcut),
                                                             C.byref(nmax), compr, shear)
        rec = {"ok": bool(ok)}
        if ok:
            rec.update(base=base.value.decode(), tag=tag.value.decode(), mech=list(mech), fire=list(fp),
                       nmin=nmin.value, mass=mass.value, fcut=fcut.value, nmax=nmax.value, compr=list(compr),
                       shear=list(shear))
        batch[name] = rec
    with open(os.path.join(MESH, "ref_batch.json"), "w") as f:
        json.dump(batch, f, indent=1, sort_keys=True)
    print("fixtures written to", MESH, "; sweep files:", sorted(os.listdir(sweep_dir)))


if __name__ == "__main__":
    main()
