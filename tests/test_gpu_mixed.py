"""Mixed-precision path (FP32 bulk, FP64 anchors + certification) vs the
FP64 oracle.  The trajectory differs from the FP64 one, so the bar is the
physics, not the bits: every returned state is certified by the canonical
FP64 force (checked here independently with the oracle), and energies agree
with the FP64 oracle's relaxed energies to a small relative tolerance."""
import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)
# Both runs stop at max|F| < 1e-10 from different trajectories.  The bar is
# 1e-10 relative to the FP64 oracle's energy, plus ten times the oracle's own
# distance from the converged minimum (its relaxation continued from that
# state to max|F| < 1e-13): on soft networks the energy at max|F| < 1e-10 is
# not settled to 1e-10 in either precision (E - E_min ~ |F|^2 / (2 lambda)
# with lambda the softest stiffness), and the mixed path must stop as close to
# the minimum as the FP64 path does, within that factor.
ENERGY_RTOL = 1e-10
UNSETTLED_FACTOR = 10.0


def energy_bar(m, x_or, e_or, fire=None):
    """Allowed |E_mixed - E_or| for the oracle state x_or of energy e_or."""
    _, _, _, r = m.fire(x_or, oracle.params(fcut=1e-13, criterion="max", **(fire or FIRE)))
    e_star = r.e_stretch + r.e_bend
    return ENERGY_RTOL * abs(e_or) + UNSETTLED_FACTOR * abs(e_or - e_star)


def batch_case(n_nets, seed, L_range=(8, 40), jitter=0.0):
    rng = np.random.default_rng(seed)
    hosts, arrs, kb, gam = [], [], [], []
    for i in range(n_nets):
        L = int(rng.integers(*L_range))
        h = nr.HostNetwork.lattice(L, L, float(rng.uniform(0.6, 0.8)), jitter, seed + i,
                                   line_triples=jitter > 0)
        if jitter == 0:
            h.get_triples()
        hosts.append(h)
        arrs.append(h.arrays())
        kb.append(float(10 ** rng.uniform(-4, -2)))
        gam.append(float(rng.uniform(0.005, 0.08)))
    return hosts, arrs, np.array(kb), np.array(gam)


@pytest.mark.parametrize("jitter", [0.0, 0.05])
def test_mixed_batch_certified_and_matches_fp64_oracle(cuda, jitter):
    hosts, arrs, kb, gam = batch_case(10, 77, jitter=jitter)
    b = nr.Batch(hosts, 1.0, kb)
    b.affine_displace(gam * (b.maxy - b.miny), 0.0)
    reps = b.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **FIRE))
    X = b.positions()
    for i, a in enumerate(arrs):
        r = reps[i]
        assert r.status == nr.NR_OK
        assert r.max_force < 1e-10 and r.fp64_steps >= 1
        x = X[b.offsets[i]:b.offsets[i + 1]]
        m = oracle.Model(a, 1.0, kb[i])
        # independent certification with the oracle's force
        assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
        es, eb = m.energies(x)
        assert es == r.e_stretch and eb == r.e_bend
        H = a["maxy"] - a["miny"]
        x0 = oracle.affine_displace(a["points"], a["miny"], H, gam[i] * H, 0.0)
        x_or, _, _, orep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max", **FIRE))
        e_or = orep.e_stretch + orep.e_bend
        assert abs(es + eb - e_or) <= energy_bar(m, x_or, e_or)
        # the anchor is re-taken rarely: FP64 evaluations are a small
        # fraction of the iterations
        assert r.fp64_steps <= max(20, r.steps // 50)


@pytest.mark.parametrize("kernel", ["grid", "tile"])
def test_mixed_single_network_grid_kernel(cuda, kernel, monkeypatch):
    """A network above the one-CTA size runs on a cooperative kernel over the
    whole GPU: the grid kernel (four passes per step) or the tiled one (one
    grid barrier per step; forced here on a small network, so its tiles are
    small and most items lie on tile boundaries)."""
    if kernel == "grid":
        monkeypatch.setenv("NR_MIX_KERNEL", "grid")
    else:
        monkeypatch.setenv("NR_TILE_MIN_NODES", "5000")
    h = nr.HostNetwork.lattice(80, 80, 0.8, 0.0, 5).get_triples()
    a = h.arrays()
    H = a["maxy"] - a["miny"]
    net = nr.Network(h, 1.0, 1e-2)
    net.affine_displace(a["miny"], H, 0.02 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **FIRE))
    assert rep.status == nr.NR_OK and rep.max_force < 1e-10
    x = net.positions()
    m = oracle.Model(a, 1.0, 1e-2)
    assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.02 * H, 0.0)
    x_or, _, _, orep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max", **FIRE))
    e_or = orep.e_stretch + orep.e_bend
    assert abs(rep.e_stretch + rep.e_bend - e_or) <= energy_bar(m, x_or, e_or)


def test_mixed_step_cap_reports_fp64_state(cuda):
    h = nr.HostNetwork.lattice(20, 20, 0.7, 0.0, 3).get_triples()
    a = h.arrays()
    H = a["maxy"] - a["miny"]
    net = nr.Network(h, 1.0, 1e-3)
    net.affine_displace(a["miny"], H, 0.05 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-12, criterion="max", precision="mixed", max_steps=50, **FIRE))
    assert rep.status == nr.NR_NOT_CONVERGED and rep.steps == 50
    # the reported force and energies are the FP64 ones at the returned positions
    x = net.positions()
    m = oracle.Model(a, 1.0, 1e-3)
    assert abs(rep.max_force - np.sqrt((m.forces(x) ** 2).sum(1)).max()) <= 1e-14 * rep.max_force
    es, eb = m.energies(x)
    assert (es, eb) == (rep.e_stretch, rep.e_bend)


@pytest.mark.parametrize("kernel,cluster,threads", [
    ("dsm", None, None), ("dsm", "1", None), ("dsm", "2", None), ("dsm", "4", "512"), ("dsm", "16", None),
    ("l2", None, None), ("l2", "4", None), ("l2", "1", "512"),
])
def test_mixed_cluster_teams(cuda, kernel, cluster, threads, monkeypatch):
    """Batches run one thread-block cluster per network: the state of a step
    in distributed shared memory ("dsm", the default when it fits) or in
    global memory ("l2"), for several cluster sizes and CTA widths; results
    certified by the oracle's FP64 force."""
    monkeypatch.setenv("NR_MIX_KERNEL", kernel)
    if cluster:
        monkeypatch.setenv("NR_CLUSTER", cluster)
    if threads:
        monkeypatch.setenv("NR_MIX_THREADS", threads)
    rng = np.random.default_rng(5)
    hosts, arrs, kb, gam = [], [], [], []
    for i, L in enumerate([50, 12, 44, 20]):
        h = nr.HostNetwork.lattice(L, L, 0.75, 0.0, 900 + i).get_triples()
        hosts.append(h)
        arrs.append(h.arrays())
        kb.append(1e-2)
        gam.append(float(rng.uniform(0.01, 0.03)))
    kb, gam = np.array(kb), np.array(gam)
    b = nr.Batch(hosts, 1.0, kb)
    b.affine_displace(gam * (b.maxy - b.miny), 0.0)
    reps = b.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **FIRE))
    X = b.positions()
    for i, a in enumerate(arrs):
        assert reps[i].status == nr.NR_OK
        x = X[b.offsets[i]:b.offsets[i + 1]]
        m = oracle.Model(a, 1.0, kb[i])
        assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
        es, eb = m.energies(x)
        assert (es, eb) == (reps[i].e_stretch, reps[i].e_bend)


@pytest.mark.parametrize("escalate", ["0", "0.5", "0.25"])
def test_mixed_escalation(cuda, escalate, monkeypatch):
    """When part of the clusters has gone idle, networks still running stop
    at an anchor and resume on clusters twice as large (NR_ESCALATE: idle
    fraction, 0 = never).  One soft network among quick stiff ones runs
    through every phase; results stay certified by the oracle's FP64 force
    and its energies."""
    monkeypatch.setenv("NR_ESCALATE", escalate)
    monkeypatch.delenv("NR_CLUSTER", raising=False)
    specs = [(30, 0.6, 1e-5, 0.05)] + [(20, 0.75, 1e-2, 0.02)] * 7
    hosts, arrs = [], []
    for i, (L, p, _, _) in enumerate(specs):
        h = nr.HostNetwork.lattice(L, L, p, 0.0, 700 + i).get_triples()
        hosts.append(h)
        arrs.append(h.arrays())
    kb = np.array([s[2] for s in specs])
    gam = np.array([s[3] for s in specs])
    b = nr.Batch(hosts, 1.0, kb)
    b.affine_displace(gam * (b.maxy - b.miny), 0.0)
    reps = b.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **FIRE))
    X = b.positions()
    assert reps[0].steps > 5 * max(r.steps for r in reps[1:])
    for i, a in enumerate(arrs):
        assert reps[i].status == nr.NR_OK
        x = X[b.offsets[i]:b.offsets[i + 1]]
        m = oracle.Model(a, 1.0, kb[i])
        assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
        assert m.energies(x) == (reps[i].e_stretch, reps[i].e_bend)


def test_mixed_mikado_certified(cuda):
    """Mixed precision on Mikado networks (per-item stiffness, wraps, very
    short segments): a batch of two, certified by the oracle's FP64 force.
    (Mikado networks whose shortest segments are stiffer than dt_max resolves
    diverge in FP64 as well; with dt_max = 0.05 sqrt(l0_min) these two
    relax in the oracle in 78K and 134K steps.)"""
    hosts = [nr.HostNetwork.mikado(300, 0.1, 1.0, 1e-3, s) for s in (7, 8)]
    arrs = [h.arrays() for h in hosts]
    dt_max = 0.05 * float(np.sqrt(min(a["edge_l0"].min() for a in arrs)))
    b = nr.Batch(hosts, 1.0, np.ones(2))
    b.affine_displace(0.01 * (b.maxy - b.miny), 0.0)
    reps = b.relax(nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **dict(FIRE, dt_max=dt_max)))
    X = b.positions()
    for i, a in enumerate(arrs):
        assert reps[i].status == nr.NR_OK
        x = X[b.offsets[i]:b.offsets[i + 1]]
        m = oracle.Model(a, 1.0, 1.0)
        assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
        assert m.energies(x) == (reps[i].e_stretch, reps[i].e_bend)


def test_sweep_graph_mixed_grid_equals_step_by_step(cuda):
    """5184 nodes: the cooperative mixed kernel, captured in one CUDA graph
    per sweep; its integer-only atomics keep it deterministic, so the graph
    and the step-by-step sweep agree bit for bit."""
    h = nr.HostNetwork.lattice(72, 72, 0.65, 0.0, 3).get_triples()
    prm = nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **FIRE)
    recs, pos = nr.Network(h, ks=1.0, kb=1e-3).sweep([0, 0, 0], [0.01, 0.02, 0.01], prm, keep_positions=True,
                                                     graph=True)
    precs, ppos = nr.Network(h, ks=1.0, kb=1e-3).sweep([0, 0, 0], [0.01, 0.02, 0.01], prm, keep_positions=True)
    key = lambda r: (r.curr_disp, r.e_stretch, r.e_bend, r.max_force, r.steps, r.fp64_steps, r.status)
    assert len(recs) == len(precs) == 2
    assert [key(r) for r in recs] == [key(r) for r in precs]
    assert all(r.status == nr.NR_OK and r.max_force < 1e-10 for r in recs)
    assert np.array_equal(pos, ppos)


@pytest.mark.parametrize("threads", ["512", "768", "256"])
@pytest.mark.parametrize("case", ["jitter", "per_item"])
def test_mixed_tile_kernel_certified(cuda, case, threads, monkeypatch):
    """The tiled kernel (one 512- or 768-thread CTA, or two 256-thread CTAs,
    per SM)
    on a jittered lattice with generator triples (rest angles), and on one
    with a stiffness per bond and per triple (random in [0.5, 2] and
    [1e-3, 1e-2], as Mikado networks have): every state certified by the
    oracle's FP64 force, energies within the bar, and the tiled sweep as one
    CUDA graph equal to the step-by-step sweep."""
    monkeypatch.setenv("NR_TILE_MIN_NODES", "1000")
    monkeypatch.setenv("NR_TILE_NODES", "128")
    monkeypatch.setenv("NR_TILE_THREADS", threads)
    h = nr.HostNetwork.lattice(70, 70, 0.8, 0.05, 17 if case == "jitter" else 19, line_triples=True)
    ks, kb, fire = 1.0, 1e-2, dict(FIRE)
    if case == "per_item":
        rng = np.random.default_rng(3)
        a0 = h.arrays()
        h.set_bond_k(rng.uniform(0.5, 2.0, len(a0["edge_l0"])))
        h.set_triples(a0["tri_hjk"], a0["tri_wrap"], kb=10 ** rng.uniform(-3, -2, len(a0["tri_hjk"])),
                      phi0=a0["tri_phi0"])
        kb = 1.0
    a = h.arrays()
    assert len(a["points"]) > 4096  # above the one-CTA size: a grid-wide kernel
    H = a["maxy"] - a["miny"]
    net = nr.Network(h, ks, kb)
    assert net.plan("mixed").startswith("k_fire_tile_mixed") and ("threads=%s" % threads) in net.plan("mixed")
    net.affine_displace(a["miny"], H, 0.02 * H, 0.0)
    prm = nr.fire_params(fcut=1e-10, criterion="max", precision="mixed", **fire)
    rep = net.relax(prm)
    assert rep.status == nr.NR_OK and rep.max_force < 1e-10
    x = net.positions()
    m = oracle.Model(a, ks, kb)
    assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
    assert m.energies(x) == (rep.e_stretch, rep.e_bend)
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.02 * H, 0.0)
    x_or, _, _, orep = m.fire(x0, oracle.params(fcut=1e-10, criterion="max", **fire))
    e_or = orep.e_stretch + orep.e_bend
    assert abs(rep.e_stretch + rep.e_bend - e_or) <= energy_bar(m, x_or, e_or, fire)
    # the sweep, captured as one graph, equals the step-by-step sweep
    net2 = nr.Network(h, ks, kb)
    r1, p1 = net2.sweep((0.0, 0.0, 0.0), (0.01, 0.02, 0.01), prm, keep_positions=True)
    net3 = nr.Network(h, ks, kb)
    r2, p2 = net3.sweep((0.0, 0.0, 0.0), (0.01, 0.02, 0.01), prm, keep_positions=True, graph=True)
    assert [(r.e_stretch, r.e_bend, r.steps) for r in r1] == [(r.e_stretch, r.e_bend, r.steps) for r in r2]
    assert all(np.array_equal(u, w) for u, w in zip(p1, p2))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_sweep_graph(cuda, precision):
    """nr_batch_sweep: the shear protocol on every network of a batch at once,
    the whole protocol as one CUDA graph (escalation decided on the device)
    and enqueued directly, against each network swept alone (FP64: the same
    bits as the oracle's sweep; mixed: certified and within the energy bar of
    the FP64 oracle's sweep)."""
    rng = np.random.default_rng(21)
    hosts, arrs, kb = [], [], []
    for i, L in enumerate([14, 40, 22, 56, 9]):
        h = nr.HostNetwork.lattice(L, L, float(rng.uniform(0.65, 0.8)), 0.0, 300 + i).get_triples()
        hosts.append(h)
        arrs.append(h.arrays())
        kb.append(float(10 ** rng.uniform(-3, -2)))
    prm = nr.fire_params(fcut=1e-10, criterion="max", precision=precision, **FIRE)
    shear = (0.01, 0.03, 0.01)
    res = {}
    for graph in (True, False):
        b = nr.Batch(hosts, 1.0, np.array(kb))
        res[graph] = (b.sweep((0.0, 0.0, 0.0), shear, prm, graph=graph), b.positions(), b.offsets)
        b.close()
    recs, X, off = res[True]
    assert len(recs) == 3
    if precision == "fp64":  # deterministic: graph and direct enqueue agree bit for bit
        recs2, X2, _ = res[False]
        assert np.array_equal(X, X2)
        assert [[(r.e_stretch, r.e_bend, r.steps) for r in s] for s in recs] == \
               [[(r.e_stretch, r.e_bend, r.steps) for r in s] for s in recs2]
    for i, a in enumerate(arrs):
        m = oracle.Model(a, 1.0, kb[i])
        H = a["maxy"] - a["miny"]
        orecs, opos, ox = m.sweep(a["points"], a["miny"], H, oracle.params(fcut=1e-10, criterion="max", **FIRE),
                                  [0.0, 0.0, 0.0], list(shear))
        x = X[off[i]:off[i + 1]]
        for k in range(3):
            r = recs[k][i]
            assert r.status == nr.NR_OK and r.is_shear == 1
            assert abs(r.curr_disp - orecs[k][0]) <= 1e-12 * H
            e_or = orecs[k][2] + orecs[k][3]
            if precision == "fp64":
                assert (r.e_stretch, r.e_bend, r.steps) == (orecs[k][2], orecs[k][3], int(orecs[k][6]))
            else:
                assert r.max_force < 1e-10
                assert abs(r.e_stretch + r.e_bend - e_or) <= energy_bar(m, opos[k], e_or)
        if precision == "fp64":
            assert np.array_equal(x, ox)
        else:
            assert np.sqrt((m.forces(x) ** 2).sum(1)).max() < 1e-10
