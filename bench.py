#!/usr/bin/env python
"""Benchmark: relaxed networks/s on the 512-network uneven batch.

Workload (config C4): 512 independent diluted triangular lattices, side
L ~ U{16..96}, bond probability p ~ U[0.55, 0.75], bending stiffness
kappa ~ logU[1e-5, 1e-2], each sheared affinely to its own gamma ~ U[0, 0.1]
and relaxed by FIRE to max|F| < 1e-10 (k = 1, Bitzek et al. FIRE
parameters).  Synthetic, seeded (network_relaxation_gb300.workloads).

One step = every network of the batch relaxed from its affinely sheared
start (positions reset from a device-resident copy), through the batched
persistent kernel (default precision: mixed FP32/FP64 with FP64
certification).  Inputs are ~0.5 GB of device data, larger than L2.

Also reported in the same JSON line:
  e2e           the same step through the public C ABI with host buffers:
                H2D of the start positions from pinned memory, relaxation,
                D2H of the relaxed positions and of the per-network reports
  roofline      the batch kernel's algorithmic bytes / its event-timed
                duration vs the measured HBM copy bandwidth; traffic = DRAM
                bytes per launch from the committed ncu summary
  energy_rel_err_vs_fp64_oracle / energy_vs_converged_fp64_minimum
                the mixed energies against the FP64 oracle's at max|F| <
                1e-10 and against its relaxation continued to 1e-12
  fp64_batched  the plain FP64 path on the same batch in one launch (the
                oracle's bits, checked), and the mixed results' errors
                against it: energy, shear stress, secant modulus, positions
  fp64          plain FP64 path, network by network, on a stratified
                sample, extrapolated by FP64 work to the batch
  c5_single_network
                one 1 048 576-node network on the tiled kernel, 1000 FIRE
                steps, with its roofline (--no-c5 skips it)
  cpu_baseline  the CPU oracle (FP64 restatement of run_fire_md) on all host
                threads, on a bounded sample of the batch plus its longest
                network timed on one thread (the makespan is the larger)
  clocks        nvidia-smi samples during the timed region
--impl reference times the CPU restatement alone (the reference's own GPU
code cannot run on this machine; its CPU path sparse_relax needs SuiteSparse).
Other workloads (--workload): C2 / C3 / C5 / M1 one large network, P3 / P5
the strain protocols as CUDA graphs (mixed and FP64), S1 the C1 sweep, L1
the linear-response solve, A1 the analyses, IO the file readers.

Multi-GPU (torchrun): --shard weak (default): every rank relaxes its own
512-network batch (seeds offset by rank), "scaling": "weak"; --shard
split: ONE batch partitioned across the ranks by expected cost,
"scaling": "strong".  No collective on the data path; value = all
networks / max-over-ranks time.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "relaxed networks/s to max|F|<1e-10 (512-network uneven batch)"
UNIT = "networks/s"


def dptr(t):
    """double* of a torch tensor's storage (host or device)."""
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def fire_params(nr, precision):
    return nr.fire_params(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10,
                          max_steps=10_000_000, criterion="max", precision=precision)


def load_c4_oracle():
    path = os.path.join(ROOT, "tests", "golden", "c4_oracle.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def mixed_bytes_per_launch(reps, hosts):
    """Algorithmic bytes of one batch launch: per node-iteration
    73 + 24 e + 12 t bytes (FP32 u, v, F read+write, fcode, bond index +
    rest vector, triple data) with e = E/N, t = T/N, times FIRE steps."""
    total = 0.0
    for r, h in zip(reps, hosts):
        i = h.info()
        total += r.steps * (73.0 * i.n_points + 24.0 * i.n_edges + 12.0 * i.n_triples)
    return total


def batch_kernel(precision, max_nodes):
    """Name of the kernel nr_batch_relax launches, by the library's policy:
    mixed precision runs one thread-block cluster of C CTAs per network, C
    the smallest power of two (at most 8) leaving at most 2304 nodes per CTA
    (NR_CLUSTER overrides), with the step's state in distributed shared
    memory (k_fire_dsm_mixed, when it fits; C4 does) or, with
    NR_MIX_KERNEL=l2, in global memory."""
    if precision != "mixed":
        return "k_fire_batch", 1
    env = os.environ.get("NR_CLUSTER")
    c = max(1, min(16, int(env))) if env else 1
    if not env:
        while c < 8 and c * 2304 < max_nodes:
            c *= 2
    if os.environ.get("NR_MIX_KERNEL") != "l2":
        return "k_fire_dsm_mixed", c
    return ("k_fire_cluster_mixed" if c > 1 else "k_fire_batch_mixed"), c


def committed_traffic(kernel):
    """DRAM bytes of one batch relaxation (all launches of `kernel` in it:
    escalation relaunches included) from the committed ncu summary
    (profiles/c4_<kernel>_dram.txt, a line 'bytes_per_launch: X'), or None."""
    path = os.path.join(ROOT, "profiles", "c4_%s_dram.txt" % kernel)
    if not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.startswith("bytes_per_launch:"):
            return float(ln.split(":", 1)[1])
    return None


def fp64_bytes_per_launch(reps, hosts):
    """FP64 algorithmic bytes: 145 + 17 e + 14 t per node-iteration."""
    total = 0.0
    for r, h in zip(reps, hosts):
        i = h.info()
        total += r.steps * (145.0 * i.n_points + 17.0 * i.n_edges + 14.0 * i.n_triples)
    return total


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(c4, n_threads, budget_s, rate_guess=8e6):
    """Stratified bounded sample of the batch for the CPU oracle: networks
    in index order, skipping any whose FP64 work alone exceeds the budget,
    until the total work fills budget_s on n_threads."""
    cap = budget_s * rate_guess
    target = budget_s * rate_guess * n_threads * 0.8
    pick, work = [], 0.0
    for i, r in enumerate(c4["networks"]):
        w = r["steps"] * r["n_points"]
        if w > cap:
            continue
        pick.append(i)
        work += w
        if work >= target:
            break
    return pick


def run_cpu_baseline(c4, n_threads, budget_s, tail_s=3.0):
    """Times the oracle on the sample and on the batch's longest network;
    returns (networks/s for the full batch, node-iterations/s, wall seconds,
    description).  The inputs come from the oracle's own restatement of the
    lattice generator, so this leg loads no product code.

    The full batch on n_threads takes at least the larger of (a) its FP64
    node-iterations at the sample's all-thread rate and (b) its longest
    network alone on one thread (a network is not split across threads).
    (b) is timed on the longest network itself, capped at about tail_s
    seconds of FIRE steps (the cost per FIRE step is constant), and scaled
    to that network's full step count.  The value is 512 / that makespan."""
    import oracle

    pick = cpu_sample(c4, n_threads, budget_s)
    rows = [c4["networks"][i] for i in pick]
    models, starts = [], []
    for r in rows:
        a = oracle.lattice_with_triples(r["L"], r["L"], r["p"], r["seed"])
        H = a["maxy"] - a["miny"]
        models.append(oracle.Model(a, 1.0, r["kappa"]))
        starts.append(oracle.affine_displace(a["points"], a["miny"], H, r["gamma"] * H, 0.0))
    prm = oracle.params(fcut=1e-10, criterion="max", max_steps=10**7)
    t = time.perf_counter()
    _, reps = oracle.fire_batch(models, starts, prm, n_threads)
    wall = time.perf_counter() - t
    work = sum(rep.steps * m.n for rep, m in zip(reps, models))
    rate = work / wall
    # the longest network on one thread, capped
    tail = max(c4["networks"], key=lambda r: r["steps"] * r["n_points"])
    a = oracle.lattice_with_triples(tail["L"], tail["L"], tail["p"], tail["seed"])
    H = a["maxy"] - a["miny"]
    m = oracle.Model(a, 1.0, tail["kappa"])
    cap = max(100, min(tail["steps"], int(tail_s * 2e7 / m.n)))
    x0 = oracle.affine_displace(a["points"], a["miny"], H, tail["gamma"] * H, 0.0)
    t = time.perf_counter()
    _, _, _, trep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max", max_steps=cap))
    t_cap = time.perf_counter() - t
    tail_makespan = t_cap * tail["steps"] / trep.steps
    throughput_makespan = c4["node_iterations"] / rate
    makespan = max(throughput_makespan, tail_makespan)
    desc = ("%d of the 512 networks (indices %d..%d, FP64 work %.2e node-iterations) on %d threads: %.3e "
            "node-iterations/s, %.0f s for the batch's %.3e; its longest network (%d nodes, %d FIRE steps) alone on "
            "one thread, %d steps timed: %.0f s; batch makespan = the larger, %.0f s"
            % (len(pick), pick[0], pick[-1], work, n_threads, rate, throughput_makespan, c4["node_iterations"],
               tail["n_points"], tail["steps"], trep.steps, tail_makespan, makespan))
    return len(c4["networks"]) / makespan, rate, wall + t_cap, desc


def reference_arm(args):
    """--impl reference: the CPU restatement of the reference's FIRE path on
    all host threads; each step a bounded sample of the batch."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    c4 = load_c4_oracle()
    n_threads = os.cpu_count() or 1
    vals, walls = [], []
    desc = ""
    for s in range(args.warmup + args.steps):
        v, rate, wall, desc = run_cpu_baseline(c4, n_threads, budget_s=args.cpu_budget)
        if s >= args.warmup:
            vals.append(v)
            walls.append(wall)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(walls)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "C4: 512 uneven diluted triangular lattices L~U{16..96}, p~U[0.55,0.75], "
                                   "kappa~logU[1e-5,1e-2], gamma~U[0,0.1], FIRE to max|F|<1e-10",
                       "parallelism": "host threads x%d" % n_threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n_threads, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU work per CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-c5", action="store_true", help="C4: skip the single-network C5 leg")
    ap.add_argument("--largest", type=int, default=0,
                    help="profiling case: only the K largest networks of the batch (not a bench line)")
    ap.add_argument("--strain-steps", type=int, default=0,
                    help="P3/P5: run the first K strain steps of the protocol (default: all)")
    ap.add_argument("--workload", default="C4",
                    choices=["C4", "C2", "C3", "C5", "M1", "L1", "A1", "IO", "S1", "P3", "P5"],
                    help="C4: the 512-network batch (the headline); C2/C3/C5: one large network on the whole GPU, "
                         "first strain increment of its protocol, FIRE steps capped by --max-steps; M1: the same "
                         "for a network embedded in a gel (network_mesh_relax.cu, FP64 path); L1: the linear-response "
                         "solve of sparse_relax.cpp on one large network; A1: the post-relaxation analyses; IO: "
                         "reading and writing network files (host only); S1: the C1 strain sweep as one CUDA graph")
    ap.add_argument("--shard", default="weak", choices=["weak", "split"],
                    help="multi-GPU layout of C4: weak (every rank its own 512-network batch) or split (ONE batch "
                         "partitioned across the ranks by longest-processing-time on N x expected iterations)")
    ap.add_argument("--reorder", default="none", choices=["none", "morton", "rcm"],
                    help="renumber every network's nodes (nr_host_network_reorder) before the batch is built")
    ap.add_argument("--side", type=int, default=0,
                    help="lattice side of the L1 workload (default 1024; a profiling case, not a bench line) or of "
                         "the P5 protocol's network (default 1024, C5; a smaller side runs the same protocol on a "
                         "smaller lattice of the same kind)")
    ap.add_argument("--fcut", type=float, default=1e-10,
                    help="C4 stop criterion max|F| < fcut of the measured precision (at most 1e-10: the metric's "
                         "criterion is met at any tighter value)")
    ap.add_argument("--dump", default="",
                    help="write the per-network reports of the last C4 relaxation to this JSON file")
    ap.add_argument("--fire-cap", type=int, default=2000,
                    help="C2/C3/C5/M1: FIRE steps of the timed relaxation (default 2000: a per-step rate)")
    ap.add_argument("--max-steps", type=int, default=10_000_000,
                    help="profiling case: FIRE step cap (networks may stop unconverged; not a bench line)")
    args = ap.parse_args()
    if not args.fcut <= 1e-10:
        ap.error("--fcut must be at most 1e-10")
    profiling_case = args.largest > 0 or args.max_steps != 10_000_000 or (args.side > 0 and args.workload == "L1")
    if profiling_case:
        args.no_cpu = args.no_fp64 = True
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "L1":
        return linear_response_arm(args)
    if args.workload == "A1":
        return analyses_arm(args)
    if args.workload == "IO":
        return io_arm(args)
    if args.workload == "S1":
        return sweep_arm(args)
    if args.workload in PROTOCOLS:
        return protocol_arm(args)
    if args.workload != "C4":
        return single_network_arm(args)

    import torch

    import network_relaxation_gb300 as nr
    from network_relaxation_gb300 import sharding, workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    split = args.shard == "split" and world > 1
    if split:
        batch_idx, prm_list = sharding.split_c4_params(rank, world)
    else:
        prm_list = sharding.rank_c4_params(rank)
        batch_idx = list(range(len(prm_list)))
    if args.largest > 0:
        prm_list = sorted(prm_list, key=lambda q: -q["L"])[:args.largest]
    hosts = workloads.c4_networks(prm_list)
    if args.reorder != "none":
        for hn in hosts:
            hn.reorder(args.reorder)
    kappa = np.array([q["kappa"] for q in prm_list])
    gamma = np.array([q["gamma"] for q in prm_list])
    batch = nr.Batch(hosts, 1.0, kappa, stream=sp)
    batch.affine_displace(gamma * (batch.maxy - batch.miny), 0.0, stream=sp)
    n_nodes = int(batch.offsets[-1])
    start_dev = torch.empty((n_nodes, 2), dtype=torch.float64, device="cuda")
    check = nr._capi.check
    lib = nr.lib()
    check(lib.nr_batch_get_positions(batch._h, dptr(start_dev), C.c_void_p(sp)), "snapshot")
    start_host = torch.empty((n_nodes, 2), dtype=torch.float64, pin_memory=True)
    start_host.copy_(start_dev)
    out_host = torch.empty_like(start_host).pin_memory()
    prm = fire_params(nr, args.precision)
    prm.max_steps = args.max_steps
    prm.fcut = args.fcut
    reps_arr = (nr.Report * batch.n)()

    def step_device():
        check(lib.nr_batch_set_positions(batch._h, dptr(start_dev), C.c_void_p(sp)), "reset")
        return lib.nr_batch_relax(batch._h, C.byref(prm), reps_arr, C.c_void_p(sp))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        check(step_device(), "warmup relax")
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kernel_ms = []
    launches = 0
    barrier()
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        check(lib.nr_batch_set_positions(batch._h, dptr(start_dev), C.c_void_p(sp)), "reset")
        k0.record(stream)
        check(lib.nr_batch_relax(batch._h, C.byref(prm), reps_arr, C.c_void_p(sp)), "relax")
        launches += lib.nr_batch_last_launches(batch._h)
        k1.record(stream)
        k1.synchronize()
        kernel_ms.append(k0.elapsed_time(k1))
    ev1.record(stream)
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms, total_nets = sharding.reduce_timing(dist, ev0.elapsed_time(ev1) / args.steps, batch.n, device="cuda")
    reps = [reps_arr[i] for i in range(batch.n)]
    value = total_nets / (ms / 1e3)

    # end to end through the C ABI with host buffers
    e2e_ms = []
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        barrier()
        t = time.perf_counter()
        check(lib.nr_batch_set_positions(batch._h, dptr(start_host), C.c_void_p(sp)), "h2d")
        check(lib.nr_batch_relax(batch._h, C.byref(prm), reps_arr, C.c_void_p(sp)), "relax")
        check(lib.nr_batch_get_positions(batch._h, dptr(out_host), C.c_void_p(sp)), "d2h")
        e2e_ms.append(1e3 * (time.perf_counter() - t))
        if not profiling_case and not all(reps_arr[i].status == 0 for i in range(batch.n)):
            raise RuntimeError("end-to-end step: a network did not converge")
    e2e_step_ms, _ = sharding.reduce_timing(dist, float(np.mean(e2e_ms)), batch.n, device="cuda")
    if args.dump and rank == 0:
        with open(args.dump, "w") as f:
            json.dump({"fcut": args.fcut, "precision": args.precision, "batch_index": batch_idx,
                       "networks": [dict(steps=r.steps, fp64_steps=r.fp64_steps, status=r.status,
                                         e_stretch=r.e_stretch.hex(), e_bend=r.e_bend.hex(), max_force=r.max_force,
                                         stress=[r.stress_xx, r.stress_yy, r.stress_xy])
                                    for r in (reps_arr[i] for i in range(batch.n))]}, f)
    h2d = n_nodes * 16
    d2h = n_nodes * 16 + batch.n * C.sizeof(nr.Report)

    steps = np.array([r.steps for r in reps])
    status = [r.status for r in reps]
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm = peaks.get("hbm_gbs")
    peak_kind = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    bytes_launch = (mixed_bytes_per_launch if args.precision == "mixed" else fp64_bytes_per_launch)(reps, hosts)
    kname, kcl = batch_kernel(args.precision, max(h.n_points for h in hosts))
    traffic = committed_traffic(kname)
    kern_ms = float(np.mean(kernel_ms))
    achieved = bytes_launch / (kern_ms / 1e3) / 1e9
    c4 = load_c4_oracle() if rank == 0 and not profiling_case else None
    line = None
    if rank == 0:
        node_iters = float(sum(r.steps * h.n_points for r, h in zip(reps, hosts)))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong" if split else "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": "C4: 512 uneven diluted triangular lattices L~U{16..96}, p~U[0.55,0.75], "
                                   "kappa~logU[1e-5,1e-2], gamma~U[0,0.1], FIRE to max|F|<1e-10",
                       "precision": args.precision, "node_order": args.reorder if args.reorder != "none" else "generator (rows)",
                       "networks_per_gpu": batch.n, "nodes_per_gpu": n_nodes,
                       "l2": "inputs larger than L2 (%.0f MB device data)" % (batch_bytes(batch) / 1e6),
                       "parallelism": ("one batch split across %d GPUs by expected cost" % world if split else
                                       "one batch per GPU" if world > 1 else "single GPU")},
            "e2e": {"value": total_nets / (e2e_step_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps, "ms_per_step": e2e_step_ms},
            "gpu_launches": launches,
            "profiling_case": ({"largest": args.largest, "max_steps": args.max_steps} if profiling_case else None),
            "node_iter_per_s": world * node_iters / (ms / 1e3),
            "iterations": {"p50": float(np.median(steps)), "p99": float(np.percentile(steps, 99)),
                           "max": int(steps.max())},
            "all_converged": all(s == 0 for s in status),
            "fp64_anchor_evals_median": float(np.median([r.fp64_steps for r in reps])),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic, "algorithmic_bytes": bytes_launch, "peak_source": peak_kind,
                         "kernel": kname, "cluster_ctas": kcl, "plan": batch.plan(args.precision)},
            "tuning_table": tuning_table_name(nr),
            "clocks": clk,
            "wall_s_timed_region": wall,
        }
        if c4 is not None and rank == 0:
            rows = [c4["networks"][i] for i in batch_idx]
            e_or = np.array([float.fromhex(r["e_stretch"]) + float.fromhex(r["e_bend"]) for r in rows])
            e_gpu = np.array([r.e_stretch + r.e_bend for r in reps])
            line["energy_rel_err_vs_fp64_oracle"] = error_stats(e_gpu, e_or, oracle_uncertainty(batch_idx))
            e_min = converged_energies(batch_idx)
            if e_min is not None:
                d_gpu = np.abs(e_gpu - e_min) / np.abs(e_min)
                d_or = np.abs(e_or - e_min) / np.abs(e_min)
                line["energy_vs_converged_fp64_minimum"] = {
                    "what": "relative distance from the FP64 oracle's energy continued to max|F| < 1e-12",
                    "this_run": error_stats(e_gpu, e_min), "fp64_oracle_at_1e-10": error_stats(e_or, e_min),
                    "n_farther_than_max_1e-10_and_oracle": int((d_gpu > np.maximum(1e-10, d_or)).sum())}
            line["fp64_node_iterations"] = c4["node_iterations"]
    if rank == 0 and not args.no_fp64 and c4 is not None and args.precision == "mixed":
        line["fp64_batched"] = fp64_batched(nr, hosts, kappa, gamma, batch_idx, c4, sp, reps, out_host.numpy(),
                                            batch.offsets, value)
    if rank == 0 and not args.no_fp64 and c4 is not None:
        line["fp64"] = fp64_network_by_network(nr, hosts, prm_list, c4, sp)
        line["batched_vs_fp64_network_by_network"] = value / line["fp64"]["value"]
    if rank == 0 and not args.no_c5 and not profiling_case:
        # the single-network kernel beside the batch: C5's first shear
        # increment, 1000 FIRE steps, W = 3
        _, us, ms5, roof5, last5, _, _, _, _ = single_network_measure(nr, torch, "C5", "mixed", 1000, 3, 1)
        line["c5_single_network"] = {
            "what": "C5: one 1 048 576-node lattice (p=0.65, jitter 0.05, seed 5), first shear increment 0.0025, "
                    "1000 FIRE steps, mixed precision, inputs larger than L2",
            "us_per_fire_step": us, "ms_per_relaxation": ms5, "roofline": roof5,
            "max_force_after_1000_steps": last5.max_force}
    if rank == 0 and not args.no_cpu and c4 is not None:
        n_threads = os.cpu_count() or 1
        v, rate, wall_cpu, desc = run_cpu_baseline(c4, n_threads, args.cpu_budget)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": n_threads, "kind": "port", "sample": desc,
                                "node_iter_per_s": rate, "wall_s": wall_cpu}
        v1, rate1, wall1, desc1 = run_cpu_baseline(c4, 1, min(5.0, args.cpu_budget))
        line["cpu_single_thread"] = {"value": v1, "unit": UNIT, "cores": 1, "kind": "port", "sample": desc1,
                                     "node_iter_per_s": rate1, "wall_s": wall1}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def oracle_uncertainty(batch_idx):
    """Per network, how far the FP64 oracle's own energy moves (relative)
    when its relaxation is continued from max|F| < 1e-10 to max|F| < 1e-12
    (tests/golden/c4_oracle_polish.json, the networks where it was
    measured), else None."""
    path = os.path.join(ROOT, "tests", "golden", "c4_oracle_polish.json")
    if not os.path.exists(path):
        return None
    pol = {r["index"]: r for r in json.load(open(path))["networks"]}
    out = []
    for i in batch_idx:
        r = pol.get(i)
        out.append(abs(r["rel_change"]) if r else None)
    return out


def converged_energies(batch_idx):
    """Per network, the FP64 oracle's energy continued to max|F| < 1e-12
    (tests/golden/c4_oracle_polish.json), or None when the fixture is
    absent."""
    path = os.path.join(ROOT, "tests", "golden", "c4_oracle_polish.json")
    if not os.path.exists(path):
        return None
    pol = {r["index"]: r for r in json.load(open(path))["networks"]}
    if any(i not in pol for i in batch_idx):
        return None
    return np.array([float.fromhex(pol[i]["e_stretch"]) + float.fromhex(pol[i]["e_bend"]) for i in batch_idx])


def error_stats(got, ref, uncertainty=None, bar=1e-10):
    """Relative errors |got - ref| / |ref|: max, p99, median, the count above
    `bar`, and (with the oracle's own per-network uncertainty) the count
    above max(bar, that uncertainty)."""
    rel = np.abs(np.asarray(got) - np.asarray(ref)) / np.abs(np.asarray(ref))
    out = {"max": float(rel.max()), "p99": float(np.percentile(rel, 99)), "median": float(np.median(rel)),
           "bar": bar, "n_above_bar": int((rel > bar).sum()), "n": int(len(rel)),
           "worst_index": int(np.argmax(rel))}
    if uncertainty is not None:
        lim = np.array([max(bar, u) if u is not None else bar for u in uncertainty])
        out["n_above_max_bar_oracle_uncertainty"] = int((rel > lim).sum())
    return out


def fp64_batched(nr, hosts, kappa, gamma, batch_idx, c4, sp, mixed_reps, mixed_pos, offsets, mixed_value):
    """The plain FP64 path on the same batch in one persistent launch
    (thread-block clusters of 8 CTAs per network, k_fire_cluster): timed
    once with CUDA events; its results are the oracle's bits (checked against
    the committed oracle run), so it is also the full FP64 reference the
    mixed results are measured against: energies, shear stress, secant
    shear modulus 2E/(gamma^2 A) and positions."""
    import torch

    b = nr.Batch(hosts, 1.0, kappa, stream=sp)
    b.affine_displace(gamma * (b.maxy - b.miny), 0.0, stream=sp)
    prm = fire_params(nr, "fp64")
    reps_arr = (nr.Report * b.n)()
    lib = nr.lib()
    plan64 = b.plan("fp64")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    nr._capi.check(lib.nr_batch_relax(b._h, C.byref(prm), reps_arr, C.c_void_p(sp)), "fp64 batch relax")
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    reps = [reps_arr[i] for i in range(b.n)]
    x64 = b.positions(stream=sp)
    rows = [c4["networks"][i] for i in batch_idx]
    same = sum(1 for r, g in zip(reps, rows) if r.steps == g["steps"] and r.e_stretch.hex() == g["e_stretch"]
               and r.e_bend.hex() == g["e_bend"])
    e64 = np.array([r.e_stretch + r.e_bend for r in reps])
    emx = np.array([r.e_stretch + r.e_bend for r in mixed_reps])
    s64 = np.array([r.stress_xy for r in reps])
    smx = np.array([r.stress_xy for r in mixed_reps])
    area = np.array([h.info().offset * (h.info().maxy - h.info().miny) for h in hosts])
    g64 = 2 * e64 / (gamma ** 2 * area)
    gmx = 2 * emx / (gamma ** 2 * area)
    dx = [float(np.sqrt(((mixed_pos[offsets[i]:offsets[i + 1]] - x64[offsets[i]:offsets[i + 1]]) ** 2).sum(1)).max())
          for i in range(b.n)]
    b.close()
    unc = oracle_uncertainty(batch_idx)
    return {"value": len(hosts) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": 1,
            "kernel": plan64, "bit_identical_to_oracle": "%d of %d" % (same, len(rows)),
            "mixed_vs_fp64_batched": mixed_value / (len(hosts) / (ms / 1e3)),
            "mixed_errors_vs_fp64": {
                "energy": error_stats(emx, e64, unc),
                "shear_stress": error_stats(smx, s64),
                "secant_shear_modulus_2E_over_gamma2_A": error_stats(gmx, g64, unc),
                "max_position_difference_lattice_spacings": {"max": float(np.max(dx)),
                                                             "p99": float(np.percentile(dx, 99)),
                                                             "median": float(np.median(dx))}}}


SINGLE = {
    # name: (generator, kappa, strain increment (shear x, compression y) of the protocol's first step)
    "C2": ("lattice 256x256, p=0.65, jitter 0.05, generator triples, seed 2", 1e-4, (0.01, 0.0)),
    "C5": ("lattice 1024x1024, p=0.65, jitter 0.05, generator triples, seed 5", 1e-4, (0.0025, 0.0)),
    "C3": ("Mikado, 15850 fibres of length 0.05, k = 1/l0, kb = kappa0/mean l0, seed 3", 1e-5, (0.0, -0.01)),
    "M1": ("network in a gel (network_mesh_relax.cu): 1024x768 grid + copy column, p=0.65, no jitter, triples by "
           "get_triples, 2 triangles per cell, seed 8; smod 0.3, bmod 1.0, dilation 0.02", 1e-4, (0.0025, 0.0)),
}
GEL_M1 = (0.3, 1.0, 0.02)


def single_network(nr, name):
    if name == "C2":
        return nr.HostNetwork.lattice(256, 256, 0.65, 0.05, 2, line_triples=True), 1e-4, 0.1
    if name == "C5":
        return nr.HostNetwork.lattice(1024, 1024, 0.65, 0.05, 5, line_triples=True), 1e-4, 0.1
    if name == "M1":
        return nr.HostNetwork.lattice_mesh(1024, 768, 0.65, 0.0, 8).get_triples(), 1e-4, 0.1
    h = nr.HostNetwork.mikado(15850, 0.05, 1.0, 1e-5, 3)
    return h, 1.0, 0.05 * float(np.sqrt(h.arrays()["edge_l0"].min()))


def mesh_cpu_baseline(h, gel, sx, sy, steps, threads=1):
    """The oracle's FP64 FIRE (gel included) on the same composite, `steps`
    iterations on one host thread: node-iterations/s."""
    import oracle

    a = h.arrays()
    m = oracle.Model(a, 1.0, SINGLE["M1"][1], gel=oracle.mesh_gel(a, *gel))
    H = a["maxy"] - a["miny"]
    x0 = oracle.affine_displace(a["points"], a["miny"], H, sx * H, sy * H)
    t0 = time.perf_counter()
    _, _, _, rep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max", max_steps=steps))
    dt = time.perf_counter() - t0
    return len(a["points"]) * rep.steps / dt, rep.steps, dt


def single_network_measure(nr, torch, workload, precision, cap, warmup, steps):
    """One large network (C2 / C3 / C5 / M1) relaxed from the first strain
    increment of its protocol, FIRE steps capped at `cap`, timed with CUDA
    events on the current stream: (node-iterations/s, us per FIRE step,
    the roofline dict, the last report, network info, gel info, plan)."""
    h, kb, dt_max = single_network(nr, workload)
    info = h.info()
    mesh = h.mesh_info()
    net = nr.Network(h, 1.0, kb)
    if workload == "M1":
        net.set_gel(*GEL_M1)
        precision = "fp64"  # gel-coupled networks relax on the FP64 path
    H = net.maxy - net.miny
    sx, sy = SINGLE[workload][2]
    net.affine_displace(net.miny, H, sx * H, sy * H)
    x0 = net.positions()
    plan = net.plan(precision)
    prm = nr.fire_params(alpha0=0.1, falpha=0.99, dt_max=dt_max, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10,
                         max_steps=cap, criterion="max", precision=precision)
    stream = torch.cuda.current_stream()
    times, fire_steps, last = [], 0, None
    for s in range(warmup + steps):
        net.set_positions(x0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rep = net.relax(prm)
        e1.record(stream)
        e1.synchronize()
        if s >= warmup:
            times.append(e0.elapsed_time(e1))
            fire_steps = rep.steps
            last = rep
    net.close()
    ms = float(np.mean(times))
    n, e, t = info.n_points, info.n_edges / info.n_points, info.n_triples / info.n_points
    g = mesh.n_facets / info.n_points if workload == "M1" else 0.0
    bpn = (145 + 17 * e + 14 * t + 168 * g) if precision == "fp64" else (73 + 24 * e + 12 * t)
    hbm = (json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
           if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None) or 6800.0
    rate = n * fire_steps / (ms / 1e3)
    achieved = bpn * rate / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": None, "kernel": plan}
    return rate, 1e3 * ms / fire_steps, ms, roof, last, info, mesh, h, precision


def single_network_arm(args):
    """--workload C2|C3|C5|M1: one large network relaxed on the whole GPU
    (the tiled kernel, or the grid kernel below its size threshold), FIRE
    steps capped: node-iterations/s.  M1 carries a gel (FP64 path)."""
    import torch

    import network_relaxation_gb300 as nr

    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    cap = min(args.max_steps, args.fire_cap)
    rate, us, ms, roof, last, info, mesh, h, precision = single_network_measure(
        nr, torch, args.workload, args.precision, cap, args.warmup, args.steps)
    extra = {}
    if args.workload == "M1" and rank == 0 and not args.no_cpu:
        sx, sy = SINGLE["M1"][2]
        cpu_rate, cpu_steps, cpu_s = mesh_cpu_baseline(h, GEL_M1, sx, sy, 20)
        extra["cpu_baseline"] = {"value": cpu_rate, "unit": "node-iterations/s", "cores": 1, "kind": "port",
                                 "sample": "the oracle's FP64 FIRE with the gel, %d iterations of the same network "
                                           "and strain step (%.1f s)" % (cpu_steps, cpu_s)}
    if rank == 0:
        n = info.n_points
        print(json.dumps({
            "metric": "node-iterations/s, one network (%s), first strain step, FIRE capped at %d steps"
                      % (args.workload, cap),
            "value": rate, "unit": "node-iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "us_per_fire_step": us, "higher_is_better": True, "scaling": "replicas",
            "relaxation": {"fire_steps": last.steps, "status": last.status, "max_force": last.max_force,
                           "energy": last.e_stretch + last.e_bend, "stress_xy": last.stress_xy},
            "vs_baseline": None, "dtype": "f32+f64" if precision == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": "%s: %s, N=%d E=%d T=%d F=%d" % (args.workload, SINGLE[args.workload][0], n,
                                                                     info.n_edges, info.n_triples, mesh.n_facets),
                       "precision": precision},
            "gpu_launches": 3 * args.steps,
            "roofline": roof,
            **extra,
        }))
    return 0


S1 = dict(L=32, p=0.65, seed=1, ks=1.0, kb=1e-3, compr=(0.0, 0.0, 0.0), shear=(0.01, 0.1, 0.01))


def sweep_arm(args):
    """--workload S1: the strain protocol of do_relaxation_run on C1 (32 x 32
    lattice, p = 0.65, k = 1, kappa = 1e-3; shear 0.01 .. 0.1 by 0.01, ten
    warm-started relaxations to max|F| < 1e-10, FP64), as one CUDA graph
    (nr_sweep_graph) and step by step (nr_sweep).  One step = the whole
    sweep from the unstrained positions; strain steps/s.  The sweep call is
    synchronous: it is timed with CUDA events on the caller's stream around
    the call.  e2e adds the H2D of the start positions from pinned memory
    and the D2H of every shear step's relaxed positions and records."""
    import torch

    import network_relaxation_gb300 as nr

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    h = nr.HostNetwork.lattice(S1["L"], S1["L"], S1["p"], 0.0, S1["seed"]).get_triples()
    info = h.info()
    net = nr.Network(h, S1["ks"], S1["kb"])
    x0 = torch.from_numpy(net.positions()).pin_memory()
    prm = fire_params(nr, "fp64")
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))

    def run(graph, keep):
        return net.sweep(S1["compr"], S1["shear"], prm, keep_positions=keep, graph=graph,
                         stream=stream.cuda_stream)

    def timed(graph, keep):
        times, recs = [], None
        for s in range(args.warmup + args.steps):
            net.set_positions(x0.numpy())
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if keep:
                net.set_positions(x0.numpy())
            recs, pos = run(graph, keep)
            e1.record(stream)
            e1.synchronize()
            if s >= args.warmup:
                times.append(e0.elapsed_time(e1))
        return float(np.mean(times)), recs

    clocks.start()
    ms_graph, recs = timed(True, False)
    clk = clocks.stop()
    ms_plain, precs = timed(False, False)
    ms_e2e, _ = timed(True, True)
    n_steps = len(recs)
    fire_steps = sum(r.steps for r in recs)
    same = [(r.e_stretch, r.e_bend, r.steps) for r in recs] == [(r.e_stretch, r.e_bend, r.steps) for r in precs]
    line = {
        "metric": "strain steps/s, C1 shear protocol (10 relaxations to max|F|<1e-10, FP64) as one CUDA graph",
        "value": n_steps / (ms_graph / 1e3), "unit": "strain steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "replicas",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "S1: lattice 32x32, p=0.65, no jitter, seed 1, triples by get_triples; ks 1, kb 1e-3; "
                               "shear 0.01 0.1 0.01; N=%d E=%d T=%d" % (info.n_points, info.n_edges, info.n_triples),
                   "l2": "inputs are 0.1 MB (L2-resident by design: a latency-bound workload)"},
        "step_by_step": {"value": n_steps / (ms_plain / 1e3), "ms_per_step": ms_plain,
                         "records_equal_to_graph": same},
        "fire_steps_per_sweep": fire_steps, "us_per_fire_step": 1e3 * ms_graph / fire_steps,
        "e2e": {"value": n_steps / (ms_e2e / 1e3), "unit": "strain steps/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": 16 * info.n_points,
                "d2h_bytes_per_step": 16 * info.n_points * n_steps + 64 * n_steps},
        "gpu_launches": 5 * n_steps * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu:
        import oracle

        a = h.arrays()
        H = a["maxy"] - a["miny"]
        t0 = time.perf_counter()
        orecs, _, _ = oracle.Model(a, S1["ks"], S1["kb"]).sweep(
            a["points"], a["miny"], H, oracle.params(fcut=1e-10, criterion="max", max_steps=10_000_000),
            list(S1["compr"]), list(S1["shear"]))
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(orecs) / dt, "unit": "strain steps/s", "cores": 1, "kind": "port",
                                "sample": "the oracle's whole sweep, %d shear steps (%.1f s)" % (len(orecs), dt)}
    print(json.dumps(line))
    return 0


# The strain protocols of configs C5 and C3 (do_relaxation_run's loops,
# large_strain_relax.cu:924-999): network, compression and shear ranges.
PROTOCOLS = {
    "P5": dict(net="C5", compr=(0.0, 0.0, 0.0), shear=(0.0025, 0.5, 0.0025),
               what="C5 network, quasi-static simple shear to gamma = 0.5 in 200 warm-started steps"),
    "P3": dict(net="C3", compr=(0.01, 0.2, 0.01), shear=(0.0, 0.0, 0.0),
               what="C3 Mikado network, uniaxial compression to 0.2 in 20 warm-started steps"),
}


def tuning_table_name(nr):
    """The launch-policy table the library loaded, relative to the
    repository when it lies inside it (None: built-in defaults)."""
    src = nr.lib().nr_tuning_source().decode()
    if not src:
        return None
    rel = os.path.relpath(os.path.realpath(src), os.path.realpath(ROOT))
    return src if rel.startswith("..") else rel


def protocol_arm(args):
    """--workload P5|P3: the strain protocol of C5 / C3 run end to end as
    one CUDA graph per precision (nr_sweep_graph: affine increment, FIRE
    relaxation to max|F| < 1e-10 (capped at --fire-cap steps), energies and
    stress per step, no host round trip), mixed precision (the tiled kernel)
    and FP64 (the grid kernel) side by side from the same start.  Reports
    both curves (energy and stress per strain step), the mixed-vs-FP64 error
    of each converged step, wall times and the mixed kernel's algorithmic
    HBM throughput.  --strain-steps K runs the protocol's first K steps."""
    import torch

    import network_relaxation_gb300 as nr

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    pr = dict(PROTOCOLS[args.workload])
    h, kb, dt_max = single_network(nr, pr["net"])
    if args.workload == "P5" and args.side > 0:  # the same protocol on a smaller lattice of the same kind
        h = nr.HostNetwork.lattice(args.side, args.side, 0.65, 0.05, 5, line_triples=True)
        pr["what"] = pr["what"].replace("C5 network", "C5-kind lattice %dx%d" % (args.side, args.side))
    info = h.info()
    compr, shear = list(pr["compr"]), list(pr["shear"])
    k = args.strain_steps
    if k > 0:  # truncate the protocol to its first k steps
        for rng in (compr, shear):
            if rng[1] > 0 and rng[2] > 0:
                n_here = int(round((rng[1] - rng[0]) / rng[2])) + 1
                take = min(n_here, k)
                rng[1] = rng[0] + (take - 1) * rng[2]
                k -= take
            elif rng[1] > 0:
                k -= 1
            if k <= 0 and rng is compr:
                shear[1] = 0.0
                break
    cap = min(args.max_steps, args.fire_cap) if args.fire_cap != 2000 else args.max_steps
    stream = torch.cuda.current_stream()
    out, plans = {}, {}
    for prec in ("mixed",) if args.no_fp64 else ("mixed", "fp64"):
        net = nr.Network(h, 1.0, kb)
        plans[prec] = net.plan(prec)
        x0 = net.positions()
        prm = nr.fire_params(alpha0=0.1, falpha=0.99, dt_max=dt_max, finc=1.1, fdec=0.5, nmin=5, mass=1.0, fcut=1e-10,
                             max_steps=cap, criterion="max", precision=prec)
        net.set_positions(x0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        recs, _ = net.sweep(compr, shear, prm, graph=True, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        out[prec] = (e0.elapsed_time(e1), recs)
        net.close()
    ms_m, rm = out["mixed"]
    ms_d, rd = out.get("fp64", (float("nan"), []))
    n = info.n_points
    bpn = 73 + 24 * info.n_edges / n + 12 * info.n_triples / n
    fire_m = sum(r.steps for r in rm)
    achieved = bpn * n * fire_m / (ms_m / 1e3) / 1e9
    hbm = (json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
           if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None) or 6800.0
    both = [(a, b) for a, b in zip(rm, rd) if a.status == 0 and b.status == 0]
    e_err = [abs((a.e_stretch + a.e_bend) - (b.e_stretch + b.e_bend)) / abs(b.e_stretch + b.e_bend) for a, b in both]
    sxy_err = [abs(a.stress_xy - b.stress_xy) / max(abs(b.stress_xy), 1e-300) for a, b in both]
    syy_err = [abs(a.stress_yy - b.stress_yy) / max(abs(b.stress_yy), 1e-300) for a, b in both]

    def curve(rs):
        return [{"strain": (r.curr_disp if r.is_shear else r.max_comp) / (info.maxy - info.miny),
                 "fire_steps": r.steps, "status": r.status, "energy": r.e_stretch + r.e_bend,
                 "stress_xy": r.stress_xy, "stress_yy": r.stress_yy} for r in rs]

    print(json.dumps({
        "metric": "strain steps/s of the %s protocol, mixed precision, one CUDA graph" % args.workload,
        "value": len(rm) / (ms_m / 1e3), "unit": "strain steps/s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": ms_m, "higher_is_better": True, "scaling": "replicas", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "%s: %s; N=%d E=%d T=%d; FIRE to max|F|<1e-10, at most %d steps per strain step"
                               % (args.workload, pr["what"], n, info.n_edges, info.n_triples, cap),
                   "strain_steps_run": len(rm), "compression": compr, "shear": shear},
        "fp64": ({"value": len(rd) / (ms_d / 1e3), "ms_per_protocol": ms_d, "fire_steps": sum(r.steps for r in rd)}
                 if rd else None),
        "mixed_fire_steps": fire_m, "us_per_fire_step_mixed": 1e3 * ms_m / max(1, fire_m),
        "us_per_fire_step_fp64": 1e3 * ms_d / max(1, sum(r.steps for r in rd)) if rd else None,
        "converged_mixed": sum(1 for r in rm if r.status == 0),
        "converged_fp64": sum(1 for r in rd if r.status == 0) if rd else None,
        "converged_both": len(both),
        "mixed_vs_fp64": {"energy_rel_max": max(e_err) if e_err else None,
                          "stress_xy_rel_max": max(sxy_err) if sxy_err else None,
                          "stress_yy_rel_max": max(syy_err) if syy_err else None},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "kernel": plans["mixed"]},
        "plan_fp64": plans.get("fp64"),
        "curve_mixed": curve(rm), "curve_fp64": curve(rd),
        "gpu_launches": 4 * (len(rm) + len(rd)),
    }))
    return 0


L1 = dict(nx=1024, ny=1024, p=0.65, seed=10, ks=1.0, kb=1e-4, mu=0.01, shear=(0.0, 0.1, 0.01))


def spr_cpu_baseline(n_side, budget_note):
    """Conjugate gradient with the same 2x2 block-Jacobi preconditioner on
    the host (scipy, one thread) for the same problem on an n_side^2
    lattice: K assembled by the oracle, the two unit loads to ||r|| <=
    1e-12 ||b||.  (The reference's SuiteSparseQR is not in this image; a
    sparse LU cannot factor these matrices, which have the floppy modes of
    isolated clusters.)"""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    import network_relaxation_gb300 as nr
    import oracle

    h = nr.HostNetwork.lattice(n_side, n_side, L1["p"], 0.0, L1["seed"])
    a = h.arrays()
    rows, cols, vals = oracle.spr_stiffness(a, L1["ks"], L1["kb"], L1["mu"])
    n = len(a["points"])
    K = sp.coo_matrix((vals, (rows, cols)), shape=(2 * n, 2 * n)).tocsr()
    K = K + sp.triu(K, 1).T
    y = a["points"][:, 1]
    free = np.repeat(~((y < a["miny"] + 1e-10) | (y > a["maxy"] - 1e-10)), 2)
    bc = np.zeros((2 * n, 2))
    bc[0::2, 1] = (y - a["miny"]) / (a["maxy"] - a["miny"])
    bc[1::2, 0] = (a["miny"] - y) / (a["maxy"] - a["miny"])
    Kff = K[free][:, free].tocsr()
    rhs = -(K[free] @ bc)
    d = Kff.diagonal()
    kxx, kyy = d[0::2], d[1::2]
    kxy = np.asarray(Kff[np.arange(0, len(d), 2), np.arange(1, len(d), 2)]).reshape(-1)
    det = kxx * kyy - kxy * kxy
    blk = (kxx > 0) & (kyy > 0) & (det > 1e-12 * kxx * kyy)
    safe = np.where(blk, det, 1.0)
    a00 = np.where(blk, kyy / safe, np.where(kxx > 0, 1.0 / np.where(kxx > 0, kxx, 1.0), 0.0))
    a11 = np.where(blk, kxx / safe, np.where(kyy > 0, 1.0 / np.where(kyy > 0, kyy, 1.0), 0.0))
    a01 = np.where(blk, -kxy / safe, 0.0)
    m = len(d)
    main = np.ravel(np.column_stack([a00, a11]))
    off = np.ravel(np.column_stack([a01, np.zeros_like(a01)]))[:-1]  # couples rows 2k and 2k + 1 only
    M = sp.diags([main, off, off], [0, 1, -1], shape=(m, m)).tocsr()
    t0 = time.perf_counter()
    for k in range(2):
        u, info = sla.cg(Kff, rhs[:, k], rtol=1e-12, atol=0.0, M=M, maxiter=100000)
        assert np.isfinite(u).all()
    dt = time.perf_counter() - t0
    return n, dt


def linear_response_arm(args):
    """--workload L1: sparse_relax.cpp's linear-response protocol on one
    1024 x 1024 lattice (p = 0.65, collinear triples, background shear):
    assembly excluded, the unit-load PCG solve plus every shear point of an
    11-point protocol (residual, energies, displacement field to the host)
    timed: node-solves/s = N x points / time."""
    import torch

    import network_relaxation_gb300 as nr

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    side = args.side or L1["nx"]
    h = nr.HostNetwork.lattice(side, side, L1["p"], 0.0, L1["seed"])
    n = h.n_points
    spr = nr.Spr(h, L1["ks"], L1["kb"], L1["mu"])
    cg_cap = args.max_steps if args.max_steps != 10_000_000 else None
    info = spr.info()
    W = info.maxx - info.minx
    pts = [s * W for s in np.arange(L1["shear"][0], L1["shear"][1] + 1e-9, L1["shear"][2])]
    host_u = torch.empty((n, 2), dtype=torch.float64).pin_memory()
    times, solve_ms, iters = [], [], 0
    stream = torch.cuda.current_stream()
    for s in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        spr.solve(affine=True, max_iter=cg_cap)
        e1.record(stream)
        for sh in pts:
            rec = nr.SprRecord()
            nr.check(spr._lib.nr_spr_point(spr._h, 0.0, float(sh), C.byref(rec),
                                           C.cast(host_u.data_ptr(), C.POINTER(C.c_double)), None), "nr_spr_point")
        e2.record(stream)
        e2.synchronize()
        if s >= args.warmup:
            times.append(e0.elapsed_time(e2))
            solve_ms.append(e0.elapsed_time(e1))
            iters = max(spr.info().iterations)
    info = spr.info()
    ms = float(np.mean(times))
    sms = float(np.mean(solve_ms))
    nnz_full = 2 * info.nnz_upper  # upper entries, both triangles (the diagonal counted twice: negligible)
    # per iteration: the matrix once (8 B value + 4 B column per nonzero); per free dof the fused pass
    # (6 double2 read, 5 written, the 2x2 block: 176 + 12 B) and the SpMV's own reads of r, z and write
    # of s (48 B)
    bytes_per_iter = 12.0 * nnz_full + 236.0 * info.n_free_dofs
    achieved = bytes_per_iter * iters / (sms / 1e3) / 1e9
    hbm = (json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
           if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None) or 6800.0
    extra = {}
    if not args.no_cpu:
        cn, cdt = spr_cpu_baseline(128, "")
        extra["cpu_baseline"] = {"value": cn * len(pts) / cdt, "unit": "node-solves/s", "cores": 1, "kind": "port",
                                 "sample": "CG with the same 2x2 block-Jacobi preconditioner in scipy (one thread), "
                                           "the two unit solves of the same problem on a 128 x 128 lattice (%.2f s); "
                                           "the reference's SuiteSparseQR is not in this image" % cdt}
    print(json.dumps({
        "metric": "node-solves/s, linear response of one network (L1: unit-load PCG + %d shear points)" % len(pts),
        "value": n * len(pts) / (ms / 1e3), "unit": "node-solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "solve_ms": sms, "cg_iterations": iters,
        "rel_residual": list(info.rel_residual), "higher_is_better": True, "scaling": "replicas",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "L1: lattice %dx%d, p=%g, no jitter, seed %d; ks %g, kb %g, mu %g; N=%d, free dofs %d, "
                               "upper nnz %d, SELL entries %d" % (side, side, L1["p"], L1["seed"], L1["ks"],
                                                                  L1["kb"], L1["mu"], n, info.n_free_dofs,
                                                                  info.nnz_upper, info.sell_entries)},
        "gpu_launches": args.steps * (1 + 5 * len(pts)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "kernel": "k_spr_pcg"},
        **extra,
    }))
    return 0


def analyses_arm(args):
    """--workload A1: bond strains, linear axial energy and non-affinity
    (strain_calc.cpp, axial_contribution.cpp, na_calc.cpp) of one
    1024 x 1024 lattice (p = 0.65) and a seeded displacement field.  One
    step = the three analyses; value on device-resident arrays, e2e with
    host arrays (copies inside the timed region)."""
    import torch

    import network_relaxation_gb300 as nr
    import oracle

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    h = nr.HostNetwork.lattice(1024, 1024, 0.65, 0.05, 12)
    a = h.arrays()
    n, e = len(a["points"]), len(a["edge_l0"])
    rng = np.random.default_rng(12)
    disp = np.ascontiguousarray(rng.normal(0.0, 0.01, (n, 2)))
    dev = torch.device("cuda:0")
    t = lambda v, dt: torch.tensor(np.ascontiguousarray(v).reshape(-1), dtype=dt, device=dev)  # noqa: E731
    d_p0, d_u = t(a["points"], torch.float64), t(disp, torch.float64)
    d_ij, d_w = t(a["edge_ij"], torch.int32), t(a["edge_wrap"], torch.int8)
    d_out = torch.empty(e, dtype=torch.float64, device=dev)
    hp = [torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in (a["points"], disp, a["edge_ij"],
                                                                           a["edge_wrap"])]
    h_out = torch.empty(e, dtype=torch.float64).pin_memory()
    lib = nr.lib()
    vp = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    res = C.c_double()
    W, miny = float(a["offset"]), float(a["miny"])

    def step(p0, u, ij, w, out):
        nr.check(lib.nr_bond_strains(n, e, W, vp(p0), vp(u), vp(ij), vp(w), vp(out), None), "nr_bond_strains")
        nr.check(lib.nr_linear_axial_energy(n, e, W, 1.0, vp(p0), vp(u), vp(ij), vp(w), C.byref(res), None),
                 "nr_linear_axial_energy")
        nr.check(lib.nr_nonaffinity(n, vp(p0), vp(u), miny, 0.0, 0.01, C.byref(res), None), "nr_nonaffinity")

    def timed(fn):
        ts = []
        for s in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            if s >= args.warmup:
                ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    ms = timed(lambda: step(d_p0, d_u, d_ij, d_w, d_out))
    ms_e2e = timed(lambda: step(hp[0], hp[1], hp[2], hp[3], h_out))
    # algorithmic bytes: per node its two xy pairs (32 B) once per analysis; per bond i, j, wrap (9 B), and the
    # strain written (8 B)
    bytes_step = 3 * 32.0 * n + 2 * 9.0 * e + 8.0 * e
    hbm = (json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
           if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None) or 6800.0
    achieved = bytes_step / (ms / 1e3) / 1e9
    extra = {}
    if not args.no_cpu:
        t0 = time.perf_counter()
        oracle.bond_strains(a, a["points"], disp)
        oracle.linear_axial_energy(a, 1.0, a["points"], disp)
        oracle.nonaffinity(a["points"], disp, miny, 0.0, 0.01)
        cdt = time.perf_counter() - t0
        extra["cpu_baseline"] = {"value": e / cdt, "unit": "bonds/s", "cores": 1, "kind": "port",
                                 "sample": "the oracle's three analyses on the same network and field (%.2f s)" % cdt}
    print(json.dumps({
        "metric": "bonds/s through bond strains + linear axial energy + non-affinity (A1)",
        "value": e / (ms / 1e3), "unit": "bonds/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "replicas", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": "A1: lattice 1024x1024, p=0.65, jitter 0.05, seed 12, "
                                                    "displacements N(0, 0.01); N=%d E=%d" % (n, e)},
        "e2e": {"value": e / (ms_e2e / 1e3), "unit": "bonds/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": int(3 * 32 * n + 2 * 9 * e), "d2h_bytes_per_step": int(8 * e + 16)},
        "gpu_launches": args.steps * 7,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "kernel": "k_bond_strains + k_tile_sums + k_final"},
        **extra,
    }))
    return 0


def io_arm(args):
    """--workload IO (host only): a 1024 x 1024 lattice (p = 0.65) written
    and read back as .dat with get_triples, and as the binary side-car; the
    M1 composite written and read back as .nmc; the oracle's getline /
    sscanf restatement of read_network + get_triples timed beside it.
    value = nodes set up per second from .dat."""
    import network_relaxation_gb300 as nr
    import oracle

    h = nr.HostNetwork.lattice(1024, 1024, 0.65, 0.05, 5)
    n = h.n_points
    d = os.environ.get("TMPDIR", "/tmp")
    dat, binp = os.path.join(d, "nr_io_bench.dat"), os.path.join(d, "nr_io_bench.bin")
    t = {}

    def clock(name, fn):
        ts = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        t[name] = float(np.median(ts))

    clock("write_dat", lambda: h.write(dat))
    clock("read_dat", lambda: nr.HostNetwork.read(dat))
    h2 = nr.HostNetwork.read(dat)
    clock("get_triples", lambda: h2.get_triples())
    clock("write_bin", lambda: h2.write_bin(binp))
    clock("read_bin", lambda: nr.HostNetwork.read_bin(binp))
    m = nr.HostNetwork.lattice_mesh(1024, 768, 0.65, 0.0, 8)  # the M1 composite (network_mesh_relax.cu's .nmc)
    nmc = os.path.join(d, "nr_io_bench.nmc")
    clock("write_nmc", lambda: m.write_mesh(nmc))
    clock("read_nmc", lambda: nr.HostNetwork.read_mesh(nmc))
    t0 = time.perf_counter()
    oracle.read_network(dat)
    t_or = time.perf_counter() - t0
    setup = t["read_dat"] + t["get_triples"]
    print(json.dumps({
        "metric": "nodes/s set up from a .dat file (read_network + get_triples), host (IO)",
        "value": n / setup, "unit": "nodes/s", "n_gpus": 0, "steps": args.steps, "warmup": 0,
        "ms_per_step": 1e3 * setup, "higher_is_better": True, "scaling": "replicas", "vs_baseline": None,
        "dtype": "text", "data": "synthetic",
        "config": {"workload": "IO: lattice 1024x1024, p=0.65, jitter 0.05, seed 5; N=%d; %d host threads"
                               % (n, os.cpu_count() or 1)},
        "seconds": t, "gpu_launches": 0,
        "cpu_baseline": {"value": n / t_or, "unit": "nodes/s", "cores": 1, "kind": "port",
                         "sample": "the oracle's getline / sscanf restatement of read_network + get_triples on the "
                                   "same file (%.2f s)" % t_or},
    }))
    return 0


def batch_bytes(batch):
    return batch.offsets[-1] * 200.0


def fp64_network_by_network(nr, hosts, prm_list, c4, sp, budget_s=20.0):
    """Plain FP64 path (nr_relax, one network at a time on the whole GPU) on
    a stratified sample (every 16th network, capped by time), extrapolated
    to the batch by its FP64 node-iterations."""
    import torch

    idx = list(range(0, len(hosts), 16))
    done, work, t_total = [], 0.0, 0.0
    prm = fire_params(nr, "fp64")
    for i in idx:
        q = prm_list[i]
        net = nr.Network(hosts[i], 1.0, q["kappa"], stream=sp)
        H = net.maxy - net.miny
        net.affine_displace(net.miny, H, q["gamma"] * H, 0.0, stream=sp)
        torch.cuda.synchronize()
        t = time.perf_counter()
        rep = net.relax(prm, stream=sp)
        t_total += time.perf_counter() - t
        work += rep.steps * net.n
        done.append(i)
        net.close()
        if t_total > budget_s:
            break
    rate = work / t_total
    per_net = c4["node_iterations"] / len(c4["networks"])
    return {"value": rate / per_net, "unit": UNIT, "node_iter_per_s": rate,
            "sample": "%d networks (every 16th, indices %s), %.1f s" % (len(done), done[:8], t_total)}


if __name__ == "__main__":
    sys.exit(main())
