"""Autotuner of the launch policy, per size class, on the GPU it runs on.

The library's launch choices (kernel variant, CTAs per network, tile size,
thresholds between kernels, threads per CTA, escalation) read named knobs
(tuning.cu): an environment variable, else the tuning table, else a built-in
default.  This module measures the candidates of each knob on synthetic
networks of each size class, with CUDA events, and writes the table the
library loads by default on that GPU model:

    python -m network_relaxation_gb300.autotune [--out PATH] [--quick] [--only CLASSES] [--merge TABLE]

(default PATH: network_relaxation_gb300/tuning/<device name>.txt, next to
libnetrelax.so).  A JSON record of every measurement goes beside it
(<PATH>.json); --merge starts from an earlier table and replaces only the
classes tuned now.  Knobs and size classes:

  FP64, one network      NR_FP64_KERNEL (dsm | l2), NR_FP64_CLUSTER (CTAs per
                         cluster), NR_FP64_CLUSTER_NODES (largest network run
                         on a cluster instead of the grid kernel): time per
                         FIRE step on lattices of 32^2 .. 181^2 nodes
  mixed, one network     NR_TILE_MIN_NODES (smallest network run on the tiled
                         kernel), NR_TILE_THREADS (512 or 768: one CTA per
                         SM, 256: two), NR_TILE_NODES (nodes per tile): time per
                         FIRE step on lattices of 128^2 .. 1024^2 nodes
  mixed, batches         NR_CLUSTER (CTAs per network in the first phase),
                         NR_ESCALATE (idle fraction that triggers escalation),
                         NR_SOLO_NODES (networks run one per CTA beside the
                         clusters): time of the 512-network uneven batch
  FP64, batches          NR_FP64_BATCH_CLUSTER: time of a 128-network
                         sample of the uneven batch, steps capped

Each candidate runs with its knobs set in the environment (which overrides
any table), after a warm-up; a knob is written only when its best candidate
beats the built-in default's measurement, otherwise the default stays.
"""
import argparse
import contextlib
import ctypes as C
import json
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)


@contextlib.contextmanager
def knobs(**kv):
    """Sets NR_* environment knobs for the duration (None: unset)."""
    old = {k: os.environ.get(k) for k in kv}
    try:
        for k, v in kv.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = str(v)
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def per_step_us(nr, torch, h, kb, precision, steps, gamma=0.02, reps=2):
    """Microseconds per FIRE step of one network relaxed `steps` steps
    (capped run) from an affinely sheared start; best of `reps`."""
    net = nr.Network(h, 1.0, kb)
    H = net.maxy - net.miny
    net.affine_displace(net.miny, H, gamma * H, 0.0)
    x0 = net.positions()
    prm = nr.fire_params(fcut=1e-14, criterion="max", precision=precision, max_steps=steps, **FIRE)
    best = None
    for r in range(reps + 1):
        net.set_positions(x0)
        torch.cuda.synchronize()
        e0, e1 = _events(torch)
        e0.record()
        rep = net.relax(prm)
        e1.record()
        e1.synchronize()
        if r > 0:  # the first run is the warm-up
            us = 1e3 * e0.elapsed_time(e1) / max(1, rep.steps)
            best = us if best is None else min(best, us)
    plan = net.plan(precision)
    net.close()
    return best, plan


def tune_fp64_single(nr, torch, log, quick):
    sides = [32, 64, 96, 128, 181] if not quick else [32, 96]
    variants = [("dsm", 16), ("dsm", 8), ("l2", 16), ("grid", 0)]
    res = {}
    for L in sides:
        h = nr.HostNetwork.lattice(L, L, 0.7, 0.0, 3).get_triples()
        for kind, c in variants:
            kv = dict(NR_FP64_CLUSTER_NODES=0) if kind == "grid" else dict(
                NR_FP64_CLUSTER_NODES=10 ** 9, NR_FP64_KERNEL=kind, NR_FP64_CLUSTER=c)
            with knobs(**kv):
                us, plan = per_step_us(nr, torch, h, 1e-3, "fp64", 1500 if L < 128 else 600)
            res[(L, kind, c)] = us
            log.append({"class": "fp64 single", "nodes": L * L, "kernel": kind, "cluster": c, "us_per_step": us,
                        "plan": plan})
    out = {}
    # cluster variant: the best summed over the classes where clusters run
    cl = [v for v in variants if v[0] != "grid"]
    best = min(cl, key=lambda v: sum(res[(L, v[0], v[1])] for L in sides))
    out["NR_FP64_KERNEL"], out["NR_FP64_CLUSTER"] = best
    # threshold: the largest class where that variant beats the grid kernel
    thr = 0
    for L in sides:
        if res[(L, best[0], best[1])] < res[(L, "grid", 0)]:
            thr = L * L
    out["NR_FP64_CLUSTER_NODES"] = thr
    return out, res


def tune_mixed_single(nr, torch, log, quick):
    sides = [128, 256, 512, 1024] if not quick else [256, 1024]
    # (threads per CTA, tile nodes): one 512- or 768-thread CTA per SM, or
    # two 256-thread CTAs per SM with smaller tiles; larger targets are cut
    # down to fit shared memory anyway
    tiles = [(512, 512), (512, 384), (768, 512), (256, 256), (256, 192)]
    res = {}
    for L in sides:
        h = nr.HostNetwork.lattice(L, L, 0.65, 0.05, 5, line_triples=True)
        with knobs(NR_MIX_KERNEL="grid", NR_TILE_MIN_NODES=10 ** 9):
            us, plan = per_step_us(nr, torch, h, 1e-4, "mixed", 1000)
        res[(L, "grid")] = us
        log.append({"class": "mixed single", "nodes": L * L, "kernel": "grid", "us_per_step": us, "plan": plan})
        for th, t in tiles:
            with knobs(NR_MIX_KERNEL=None, NR_TILE_MIN_NODES=1, NR_TILE_THREADS=th, NR_TILE_NODES=t):
                us, plan = per_step_us(nr, torch, h, 1e-4, "mixed", 1000)
            res[(L, "tile", th, t)] = us
            log.append({"class": "mixed single", "nodes": L * L, "kernel": "tile", "threads": th, "tile_nodes": t,
                        "us_per_step": us, "plan": plan})
    out = {}
    big = sides[-1]
    best = min(tiles, key=lambda v: res[(big, "tile") + v])
    out["NR_TILE_THREADS"], out["NR_TILE_NODES"] = best
    thr = None
    for L in sides:
        if res[(L, "tile") + best] < res[(L, "grid")]:
            thr = L * L if thr is None else thr
        else:
            thr = None  # the tiled kernel must win from its threshold upwards
    out["NR_TILE_MIN_NODES"] = thr if thr is not None else 10 ** 9
    return out, res


def batch_time_ms(nr, torch, hosts, kappa, gamma, precision, max_steps=10_000_000):
    b = nr.Batch(hosts, 1.0, kappa)
    b.affine_displace(gamma * (b.maxy - b.miny), 0.0)
    x0 = b.positions()
    prm = nr.fire_params(fcut=1e-10, criterion="max", precision=precision, max_steps=max_steps, **FIRE)
    b.set_positions(x0)
    torch.cuda.synchronize()
    e0, e1 = _events(torch)
    e0.record()
    b.relax(prm)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    b.close()
    return ms


def tune_mixed_batch(nr, torch, log, quick):
    from . import workloads

    prm = workloads.c4_params()
    if quick:
        prm = prm[::4]
    hosts = workloads.c4_networks(prm)
    kappa = np.array([q["kappa"] for q in prm])
    gamma = np.array([q["gamma"] for q in prm])
    batch_time_ms(nr, torch, hosts, kappa, gamma, "mixed")  # warm-up
    default = dict(NR_CLUSTER=None, NR_ESCALATE=None, NR_SOLO_NODES=None)
    with knobs(**default):
        base = batch_time_ms(nr, torch, hosts, kappa, gamma, "mixed")
    log.append({"class": "mixed batch", "knobs": "defaults", "ms": base})
    cands = []
    for c in (2, 4, 8):
        for esc in (0.25, 0.5):
            for solo in (1024, 2304):
                cands.append(dict(NR_CLUSTER=c, NR_ESCALATE=esc, NR_SOLO_NODES=solo))
    if quick:
        cands = cands[::3]
    best, best_ms = None, base
    for kv in cands:
        with knobs(**kv):
            ms = batch_time_ms(nr, torch, hosts, kappa, gamma, "mixed")
        log.append({"class": "mixed batch", "knobs": kv, "ms": ms})
        if ms < best_ms:
            best, best_ms = kv, ms
    return (best or {}), {"default_ms": base, "best_ms": best_ms}


def tune_fp64_batch(nr, torch, log, quick):
    from . import workloads

    prm = workloads.c4_params()[::4 if not quick else 16]
    hosts = workloads.c4_networks(prm)
    kappa = np.array([q["kappa"] for q in prm])
    gamma = np.array([q["gamma"] for q in prm])
    cap = 50_000
    batch_time_ms(nr, torch, hosts, kappa, gamma, "fp64", cap)  # warm-up
    with knobs(NR_FP64_BATCH_CLUSTER=None):
        base = batch_time_ms(nr, torch, hosts, kappa, gamma, "fp64", cap)
    log.append({"class": "fp64 batch", "knobs": "defaults", "ms": base, "networks": len(hosts), "step_cap": cap})
    best, best_ms = None, base
    for c in (4, 8, 16):
        with knobs(NR_FP64_BATCH_CLUSTER=c):
            ms = batch_time_ms(nr, torch, hosts, kappa, gamma, "fp64", cap)
        log.append({"class": "fp64 batch", "knobs": {"NR_FP64_BATCH_CLUSTER": c}, "ms": ms})
        if ms < best_ms:
            best, best_ms = {"NR_FP64_BATCH_CLUSTER": c}, ms
    return (best or {}), {"default_ms": base, "best_ms": best_ms}


def default_table_path(torch):
    name = re.sub(r"[^a-z0-9]", "_", torch.cuda.get_device_name(0).lower())
    return os.path.join(HERE, "tuning", name + ".txt")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default="")
    ap.add_argument("--quick", action="store_true", help="fewer size classes and candidates")
    ap.add_argument("--only", default="", help="comma-separated subset: fp64,mixed,batch,fp64batch")
    ap.add_argument("--merge", default="",
                    help="start from this table (its .json record): the classes tuned now replace their entries")
    args = ap.parse_args(argv)
    import torch

    sys.path.insert(0, os.path.dirname(HERE))
    import network_relaxation_gb300 as nr

    # measure against the built-in defaults, not a table loaded earlier
    empty = os.path.join(os.environ.get("TMPDIR", "/tmp"), "nr_empty_tuning.txt")
    open(empty, "w").close()
    nr._capi.check(nr.lib().nr_tuning_load(empty.encode()), "nr_tuning_load")
    only = set(args.only.split(",")) if args.only else {"fp64", "mixed", "batch", "fp64batch"}
    log, table, summary = [], {}, {}
    if args.merge:
        with open(args.merge + ".json") as f:
            prev = json.load(f)
        table, summary, log = dict(prev["table"]), dict(prev["summary"]), list(prev["measurements"])
        tuned = {"fp64": "fp64 single", "mixed": "mixed single", "batch": "mixed batch", "fp64batch": "fp64 batch"}
        log = [m for m in log if m.get("class") not in {tuned[k] for k in only}]
    t0 = time.time()
    if "fp64" in only:
        out, _ = tune_fp64_single(nr, torch, log, args.quick)
        table.update(out)
    if "mixed" in only:
        out, _ = tune_mixed_single(nr, torch, log, args.quick)
        table.update(out)
    if "batch" in only:
        out, s = tune_mixed_batch(nr, torch, log, args.quick)
        table.update(out)
        summary["mixed batch"] = s
    if "fp64batch" in only:
        out, s = tune_fp64_batch(nr, torch, log, args.quick)
        table.update(out)
        summary["fp64 batch"] = s
    path = args.out or default_table_path(torch)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write("# launch-policy table written by network_relaxation_gb300.autotune on %s (%s), %.0f s\n"
                % (torch.cuda.get_device_name(0), time.strftime("%Y-%m-%d"), time.time() - t0))
        f.write("# NAME value; an environment variable of the same name overrides an entry\n")
        for k in sorted(table):
            f.write("%s %s\n" % (k, table[k]))
    with open(path + ".json", "w") as f:
        json.dump({"table": table, "summary": summary, "measurements": log}, f, indent=1, default=str)
    print(json.dumps({"table": path, "entries": table, "summary": summary}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
