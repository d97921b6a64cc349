"""Regenerates the golden fixtures in this directory from the reference's own
code (large_strain_relax.cu compiled for the host by oracle/build_ref.sh).

Run where the reference checkout exists:
    python tests/golden/make_golden.py

Fixtures (inputs are this project's seeded generators; outputs are the
reference's):
  c1.dat            32x32 triangular lattice, p=0.65, seed 1 (config C1)
  small.dat         12x12, p=0.7, seed 3
  edge_cases/*.dat  reader edge cases (blank lines, extra tokens, short
                    files, bad indices, negative y)
  ref_c1.npz        reference read_network / get_triples arrays of c1.dat,
                    fcodes, the affine start of one 0.01 shear step, and
                    run_fire_md's relaxed positions, report and step count
                    (RMS criterion, fcut = 1e-10/sqrt(2N))
  ref_readers.json  read_network's accept / reject and sizes per edge case
  ref_sweep/        do_relaxation_run outputs for small.dat: log (without the
                    elapsed-time line), edata and .pos files of a two-step
                    compression + three-step shear protocol
  ref_batch.json    parse_batch_file's results on the batch files below
"""
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

FIRE = [0.1, 0.99, 0.1, 1.1, 0.5]

EDGE_CASES = {
    "blank_lines.dat": "3 2 4.0\n\n0.0 0.0\n# not a point\n1.0 0.5\n\n2.0 1.0\n0 1 0\n\n1 2 0\n",
    "extra_tokens.dat": "3 2 4.0 extra\n0.0 0.0 9.9\n1.0 0.5\n2.0 1.0\n0 1 0 7\n1 2 -1\n",
    "too_few_points.dat": "4 1 4.0\n0.0 0.0\n1.0 0.5\n",
    "too_few_edges.dat": "3 3 4.0\n0.0 0.0\n1.0 0.5\n2.0 1.0\n0 1 0\n1 2 0\n",
    "bad_index.dat": "3 2 4.0\n0.0 0.0\n1.0 0.5\n2.0 1.0\n0 1 0\n1 3 0\n",
    "bad_header.dat": "3 -1 4.0\n0.0 0.0\n1.0 0.5\n2.0 1.0\n",
    "negative_y.dat": "4 3 10.0\n0.0 -3.0\n1.0 -2.0\n2.0 -1.0\n3.0 -2.5\n0 1 0\n1 2 0\n2 3 1\n",
    "no_trailing_newline.dat": "3 2 4.0\n0.0 0.0\n1.0 0.0\n2.0 0.0\n0 1 0\n1 2 0",
    "collinear.dat": "5 4 10.0\n0.0 0.0\n1.0 0.0\n2.0 0.0\n1.0 1.0\n1.0 -1.0\n0 1 0\n1 2 0\n3 1 0\n1 4 0\n",
    "wrapped.dat": "4 4 4.0\n0.5 0.0\n1.5 0.0\n2.5 0.0\n3.5 0.0\n0 1 0\n1 2 0\n2 3 0\n3 0 1\n",
}

BATCH_FILES = {
    "ok.txt": "# comment\n\nnet tagA\n1.0 0.001\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-10 100000\n0 0 0\n0.01 0.1 0.01\n",
    "too_few_fire.txt": "net\n1.0 0.001\n0.1 0.99 0.1\n5 1.0 1e-10 100000\n0 0 0\n0.01 0.1 0.01\n",
    "bad_range.txt": "net\n1.0 0.001\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-10 100000\n0 0 0\n0.1 0.01 0.01\n",
    "negative_k.txt": "net\n-1.0 0.001\n0.1 0.99 0.1 1.1 0.5\n5 1.0 1e-10 100000\n0 0 0\n0.01 0.1 0.01\n",
    "truncated.txt": "net\n1.0 0.001\n",
}


def main():
    if oracle.build_ref() is None:
        sys.exit("the reference checkout is not available; fixtures cannot be regenerated")
    os.makedirs(os.path.join(HERE, "edge_cases"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "batch_files"), exist_ok=True)
    nr.HostNetwork.lattice(32, 32, 0.65, 0.0, 1).write(os.path.join(HERE, "c1.dat"))
    nr.HostNetwork.lattice(12, 12, 0.7, 0.0, 3).write(os.path.join(HERE, "small.dat"))

    readers = {}
    for name, text in EDGE_CASES.items():
        path = os.path.join(HERE, "edge_cases", name)
        with open(path, "w") as f:
            f.write(text)
        ok, a = oracle.ref_read_network(path)
        readers[name] = {"ok": ok, "n_points": len(a["points"]), "n_edges": len(a["edge_l0"]),
                         "n_triples": len(a["tri_hjk"]), "points": a["points"].tolist(),
                         "edge_ij": a["edge_ij"].tolist(), "edge_l0": [float(v).hex() for v in a["edge_l0"]],
                         "edge_wrap": a["edge_wrap"].tolist(), "tri_hjk": a["tri_hjk"].tolist(),
                         "tri_wrap": a["tri_wrap"].tolist(), "miny": float(a["miny"]).hex(),
                         "maxy": float(a["maxy"]).hex(), "offset": a["offset"]}
    with open(os.path.join(HERE, "ref_readers.json"), "w") as f:
        json.dump(readers, f, indent=1)

    ok, a = oracle.ref_read_network(os.path.join(HERE, "c1.dat"))
    assert ok
    N = len(a["points"])
    H = a["maxy"] - a["miny"]
    y = a["points"][:, 1]
    fc = np.where((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10), 0, 3).astype(np.uint8)
    x0 = oracle.ref_affine_displace(a["points"], a["miny"], H, 0.01 * H, 0.0)
    fcut = 1e-10 / np.sqrt(2 * N)
    xr, rep, steps = oracle.ref_run_fire_md(a, x0, 1.0, 1e-3, fc, FIRE, 1.0, fcut, 10**6, 5)
    np.savez_compressed(os.path.join(HERE, "ref_c1.npz"), points=a["points"], edge_ij=a["edge_ij"],
                        edge_l0=a["edge_l0"], edge_wrap=a["edge_wrap"], tri_hjk=a["tri_hjk"], tri_wrap=a["tri_wrap"],
                        offset=a["offset"], miny=a["miny"], maxy=a["maxy"], fcodes=fc, x_affine=x0,
                        x_relaxed=xr, report=np.array(rep), steps=steps, fcut=fcut)

    sweep_dir = os.path.join(HERE, "ref_sweep")
    shutil.rmtree(sweep_dir, ignore_errors=True)
    os.makedirs(sweep_dir)
    small = os.path.join(HERE, "small.dat")
    L = oracle.ref_lib()
    fp = np.array(FIRE)
    compr = np.array([0.01, 0.02, 0.01])
    shear = np.array([0.01, 0.03, 0.01])
    L.ref_do_relaxation_run(small.encode(), os.path.join(sweep_dir, "small_log.txt").encode(),
                            os.path.join(sweep_dir, "small_edata.txt").encode(),
                            os.path.join(sweep_dir, "small").encode(), 1.0, 1e-3, oracle._d(fp), 5, 1.0, 1e-12,
                            10**6, oracle._d(compr), oracle._d(shear))
    with open(os.path.join(sweep_dir, "small_log.txt")) as f:
        lines = [ln for ln in f if not ln.startswith("Elapsed time")]
    with open(os.path.join(sweep_dir, "small_log.txt"), "w") as f:
        f.writelines(lines)

    import ctypes as C
    batch = {}
    for name, text in BATCH_FILES.items():
        path = os.path.join(HERE, "batch_files", name)
        with open(path, "w") as f:
            f.write(text)
        base, tag = C.create_string_buffer(1024), C.create_string_buffer(256)
        ks, kb, mass, fcut_ = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        nmin, nmax = C.c_int(), C.c_int()
        fpv, cr, sh = (C.c_double * 5)(), (C.c_double * 3)(), (C.c_double * 3)()
        ok = L.ref_parse_batch_file(path.encode(), base, 1024, tag, 256, C.byref(ks), C.byref(kb), fpv,
                                    C.byref(nmin), C.byref(mass), C.byref(fcut_), C.byref(nmax), cr, sh)
        batch[name] = {"ok": bool(ok)}
        if ok:
            batch[name].update(base=base.value.decode(), tag=tag.value.decode(), ks=ks.value, kb=kb.value,
                               fire=list(fpv), nmin=nmin.value, mass=mass.value, fcut=fcut_.value, nmax=nmax.value,
                               compr=list(cr), shear=list(sh))
    with open(os.path.join(HERE, "ref_batch.json"), "w") as f:
        json.dump(batch, f, indent=1)
    print("golden fixtures written; c1: %d steps, report %s" % (steps, rep))


if __name__ == "__main__":
    main()
