"""Regenerates the linear-response fixtures in tests/golden/spr/ from the
reference's own sparse_relax.cpp (compiled for the host by
oracle/build_ref.sh into oracle/_ref/libspr_ref.so, with dense stand-ins for
CHOLMOD / SPQR, which are absent here).

Run where the reference checkout exists:
    python tests/golden/make_spr_golden.py

Fixtures (inputs from this project's seeded generator; outputs the
reference's):
  spr/s1.dat            10 x 8 triangular lattice, p = 0.8, no jitter, seed 4
                        (collinear triples for the bending term)
  spr/s2.dat            12 x 10, p = 0.75, jitter 0.05, seed 6
  spr/ref_spr.npz       for s1 and s2: get_sparse_stiffness_mat triplets at
                        three (ks, kb, mu); the linearised energies of a
                        seeded displacement field
  spr/ref_sweep_*/      do_relaxation_run on s1.dat (ks 1, kb 1e-2, mu 0.05,
                        compression 0..0.02 by 0.01, shear 0..0.03 by 0.01,
                        strain mode, itemized): affine and top-only loading;
                        log (without the elapsed-time line), energies and
                        .disp files
  spr/ref_batch.json    parse_batch_file's results on spr/batch_files/
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

SPR = os.path.join(HERE, "spr")
CASES = [(1.0, 0.0, 0.0), (1.0, 1e-2, 0.0), (0.5, 0.1, 0.05)]
SWEEP = dict(ks=1.0, kb=1e-2, mu=0.05, compr=[0.0, 0.02, 0.01], shear=[0.0, 0.03, 0.01], strain_mode=1, itemize=1)
BATCH_FILES = {
    "ok.txt": "# linear response\n\nnet tagB\n\n1.0 0.01 0.05\n0 0.02 0.01\n# shear\n0 0.03 0.01\n",
    "no_tag.txt": "net\n1.0 0.0 0.0\n0 0 0\n0 0.1 0.05\n",
    "bad_mech.txt": "net\n1.0 0.01\n0 0 0\n0 0.1 0.05\n",
    "negative_mu.txt": "net\n1.0 0.01 -1\n0 0 0\n0 0.1 0.05\n",
    "bad_shear.txt": "net\n1.0 0.01 0.0\n0 0 0\n0.1 0.05 0.01\n",
    "truncated.txt": "net\n1.0 0.01 0.0\n0 0 0",
}


def main():
    if oracle.build_ref() is None or oracle.ref_spr_lib() is None:
        sys.exit("the reference checkout is needed to regenerate these fixtures")
    os.makedirs(os.path.join(SPR, "batch_files"), exist_ok=True)
    nr.HostNetwork.lattice(10, 8, 0.8, 0.0, 4).write(os.path.join(SPR, "s1.dat"))
    nr.HostNetwork.lattice(12, 10, 0.75, 0.05, 6).write(os.path.join(SPR, "s2.dat"))
    out = {}
    for name in ("s1", "s2"):
        r = oracle.RefSpr(os.path.join(SPR, name + ".dat"))
        assert r.ok
        for c, (ks, kb, mu) in enumerate(CASES):
            rows, cols, vals = r.stiffness(ks, kb, mu)
            out["%s_K%d_rows" % (name, c)] = rows
            out["%s_K%d_cols" % (name, c)] = cols
            out["%s_K%d_vals" % (name, c)] = vals
        u = np.random.default_rng(5).normal(size=2 * len(r.a["points"]))
        out[name + "_u"] = u
        out[name + "_energies"] = np.array(r.energies(1.0, 1e-2, 0.05, u))
    np.savez_compressed(os.path.join(SPR, "ref_spr.npz"), **out)

    S = SWEEP
    dbl = lambda v: (C.c_double * len(v))(*v)  # noqa: E731
    for affine in (1, 0):
        d = os.path.join(SPR, "ref_sweep_%s" % ("affine" if affine else "top"))
        shutil.rmtree(d, ignore_errors=True)
        os.makedirs(d)
        oracle.ref_spr_lib().ref_spr_do_relaxation_run(
            os.path.join(SPR, "s1.dat").encode(), os.path.join(d, "log.txt").encode(), os.path.join(d, "s1").encode(),
            os.path.join(d, "energies.txt").encode(), S["ks"], S["kb"], S["mu"], dbl(S["compr"]), dbl(S["shear"]),
            S["strain_mode"], affine, S["itemize"])
        log = os.path.join(d, "log.txt")
        lines = [ln for ln in open(log) if not ln.startswith("Elapsed time")]
        with open(log, "w") as f:
            f.writelines(lines)
        with open(os.path.join(d, "params.json"), "w") as f:
            json.dump({**S, "affine": affine}, f, indent=1)

    batch = {}
    for name, text in BATCH_FILES.items():
        path = os.path.join(SPR, "batch_files", name)
        with open(path, "w") as f:
            f.write(text)
        base, tag = C.create_string_buffer(1024), C.create_string_buffer(256)
        mech, c, s = (C.c_double * 3)(), (C.c_double * 3)(), (C.c_double * 3)()
        ok = oracle.ref_spr_lib().ref_spr_parse_batch_file(path.encode(), base, 1024, tag, 256, mech, c, s)
        rec = {"ok": bool(ok)}
        if ok:
            rec.update(base=base.value.decode(), tag=tag.value.decode(), mech=list(mech), compr=list(c), shear=list(s))
        batch[name] = rec
    with open(os.path.join(SPR, "ref_batch.json"), "w") as f:
        json.dump(batch, f, indent=1, sort_keys=True)
    print("fixtures written to", SPR, sorted(os.listdir(SPR)))


if __name__ == "__main__":
    main()
