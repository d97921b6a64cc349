"""FP64 oracle results for the 512-network uneven batch (config C4):
per network the FIRE step count, energies and final max|F| at
max|F| < 1e-10, written to c4_oracle.json.  The plain FP64 GPU path must
reproduce the step counts and energies exactly; the mixed path is compared
to the energies; the benchmark uses sum(steps * N) as the workload's FP64
node-iteration count.  CPU only (about 15 minutes on 8 cores):
    python tests/golden/make_c4_oracle.py [threads]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from network_relaxation_gb300 import workloads  # noqa: E402


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count()
    prm = workloads.c4_params()
    hosts = workloads.c4_networks(prm)
    models, starts = [], []
    for q, h in zip(prm, hosts):
        a = h.arrays()
        H = a["maxy"] - a["miny"]
        models.append(oracle.Model(a, 1.0, q["kappa"]))
        starts.append(oracle.affine_displace(a["points"], a["miny"], H, q["gamma"] * H, 0.0))
    t = time.time()
    xs, reps = oracle.fire_batch(models, starts, oracle.params(fcut=1e-10, criterion="max", max_steps=10**7), threads)
    wall = time.time() - t
    rows = []
    for q, m, r in zip(prm, models, reps):
        rows.append(dict(q, n_points=m.n, n_edges=int(m.m.n_edges), n_triples=int(m.m.n_triples), steps=r.steps,
                         converged=r.converged, e_stretch=r.e_stretch.hex(), e_bend=r.e_bend.hex(),
                         max_force=r.max_force))
    work = sum(r["steps"] * r["n_points"] for r in rows)
    out = {"fcut": 1e-10, "criterion": "max", "threads": threads, "wall_s": wall,
           "node_iterations": work, "networks": rows}
    with open(os.path.join(HERE, "c4_oracle.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("C4 oracle: %d networks, %.3e node-iterations, %.0f s on %d threads" % (len(rows), work, wall, threads))


if __name__ == "__main__":
    main()
