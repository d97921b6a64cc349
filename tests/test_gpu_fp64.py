"""FP64 GPU path vs the oracle.

The FP64 kernels use the oracle's canonical arithmetic (explicit fma, fixed
summation order, polynomial atan2), so forces, trajectories, step counts and
energies must agree BIT-FOR-BIT - a stronger bar than the 1e-10 relative
energy / 1e-8 position tolerance against the reference itself (pinned in
test_oracle_vs_reference.py).
"""
import numpy as np
import pytest

import network_relaxation_gb300 as nr
import oracle

pytestmark = pytest.mark.gpu

FIRE = dict(alpha0=0.1, falpha=0.99, dt_max=0.1, finc=1.1, fdec=0.5, nmin=5, mass=1.0)


def lattice(n, p, seed, kb=1e-3, jitter=0.0, line_triples=False):
    h = nr.HostNetwork.lattice(n, n, p, jitter, seed, line_triples=line_triples)
    if not line_triples and kb > 0:
        h.get_triples()
    return h, h.arrays()


@pytest.mark.parametrize("n,p,seed,kb", [(8, 0.65, 1, 1e-3), (32, 0.65, 1, 1e-3), (20, 0.8, 5, 0.0), (40, 0.55, 3, 1e-2)])
def test_forces_bitwise(cuda, n, p, seed, kb):
    h, a = lattice(n, p, seed, kb)
    net = nr.Network(h, ks=1.0, kb=kb)
    rng = np.random.default_rng(seed)
    x = a["points"] + rng.normal(scale=0.05, size=a["points"].shape)
    net.set_positions(x)
    F = net.forces()
    Fo = oracle.Model(a, 1.0, kb).forces(x)
    assert np.array_equal(F, Fo), np.abs(F - Fo).max()
    es, eb = net.energies()
    eso, ebo = oracle.Model(a, 1.0, kb).energies(x)
    assert es == eso and eb == ebo


def test_forces_jittered_generator_triples(cuda):
    h, a = lattice(24, 0.7, 2, jitter=0.05, line_triples=True)
    assert a["tri_phi0"] is not None and len(a["tri_hjk"]) > 0
    net = nr.Network(h, ks=1.0, kb=1e-4)
    m = oracle.Model(a, 1.0, 1e-4)
    # rest state is force-free by construction
    assert np.abs(m.forces(a["points"])[:, :]).max() < 1e-15
    x = a["points"] + np.random.default_rng(0).normal(scale=0.03, size=a["points"].shape)
    net.set_positions(x)
    assert np.array_equal(net.forces(), m.forces(x))


def test_affine_bitexact(cuda):
    h, a = lattice(16, 0.65, 4)
    net = nr.Network(h, ks=1.0, kb=1e-3)
    H = a["maxy"] - a["miny"]
    net.affine_displace(a["miny"], H, 0.013 * H, 0.0)
    net.affine_displace(a["miny"], H, 0.0, -0.007 * H)
    x = oracle.affine_displace(a["points"], a["miny"], H, 0.013 * H, 0.0)
    x = oracle.affine_displace(x, a["miny"], H, 0.0, -0.007 * H)
    assert np.array_equal(net.positions(), x)


@pytest.fixture(params=["dsm16", "dsm4", "l2_16", "grid"])
def fp64_kernel(request, monkeypatch):
    """The single-network FP64 kernel: one thread-block cluster of 16 or 4
    CTAs with the step's state in distributed shared memory (the default for
    small networks), a cluster of 16 with the state in global memory, or the
    cooperative grid kernel (software grid barriers).  The same bits."""
    kind, _, c = request.param.partition("_") if "_" in request.param else (request.param[:3], "", request.param[3:])
    if request.param == "grid":
        monkeypatch.setenv("NR_FP64_CLUSTER_NODES", "0")
    else:
        monkeypatch.setenv("NR_FP64_CLUSTER_NODES", "100000000")
        monkeypatch.setenv("NR_FP64_CLUSTER", c)
        monkeypatch.setenv("NR_FP64_KERNEL", "l2" if kind == "l2" else "dsm")
    return request.param


@pytest.mark.parametrize("crit", ["rms", "max"])
def test_relax_bitwise_c1(cuda, crit, fp64_kernel):
    """32x32, p=0.65, kappa=1e-3: one shear increment of 0.01, relaxed."""
    h, a = lattice(32, 0.65, 1)
    N = len(a["points"])
    H = a["maxy"] - a["miny"]
    fcut = 1e-10 / np.sqrt(2 * N) if crit == "rms" else 1e-10
    net = nr.Network(h, ks=1.0, kb=1e-3)
    net.affine_displace(a["miny"], H, 0.01 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=fcut, criterion=crit, **FIRE))
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.01 * H, 0.0)
    xo, vo, Fo, orep = oracle.Model(a, 1.0, 1e-3).fire(x0, oracle.params(fcut=fcut, criterion=crit, **FIRE))
    assert rep.status == nr.NR_OK
    assert rep.steps == orep.steps
    assert np.array_equal(net.positions(), xo)
    assert rep.e_stretch == orep.e_stretch and rep.e_bend == orep.e_bend
    assert rep.rms_force == orep.rms_force and rep.max_force == orep.max_force


def test_step_cap_reports_not_converged(cuda, fp64_kernel):
    h, a = lattice(16, 0.65, 2)
    net = nr.Network(h, ks=1.0, kb=1e-3)
    H = a["maxy"] - a["miny"]
    net.affine_displace(a["miny"], H, 0.05 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-12, max_steps=7, **FIRE))
    assert rep.status == nr.NR_NOT_CONVERGED and rep.steps == 7
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.05 * H, 0.0)
    xo, _, _, orep = oracle.Model(a, 1.0, 1e-3).fire(x0, oracle.params(fcut=1e-12, max_steps=7, **FIRE))
    assert np.array_equal(net.positions(), xo)


@pytest.mark.parametrize("team", ["1", "4", "16", "8-l2"])
def test_batch_equals_oracle(cuda, team, monkeypatch):
    """Uneven batch: every network bit-identical to its oracle run, with one
    CTA per network (k_fire_batch), with thread-block clusters of 4 and 16
    CTAs per network holding the state in distributed shared memory
    (k_fire_dsm64), and with clusters of 8 holding it in global memory
    (k_fire_cluster)."""
    c, _, kind = team.partition("-")
    monkeypatch.setenv("NR_FP64_BATCH_CLUSTER", c)
    monkeypatch.setenv("NR_FP64_KERNEL", kind or "dsm")
    hosts, arrs, gam = [], [], []
    rng = np.random.default_rng(11)
    for i in range(12):
        L = int(rng.integers(8, 40))
        h, a = lattice(L, float(rng.uniform(0.6, 0.8)), 100 + i)
        hosts.append(h)
        arrs.append(a)
        gam.append(float(rng.uniform(0.005, 0.05)))
    kbs = [1e-3] * len(hosts)
    b = nr.Batch(hosts, ks=1.0, kb=kbs)
    H = b.maxy - b.miny
    b.affine_displace(np.array(gam) * H, 0.0)
    prm = nr.fire_params(fcut=1e-10, criterion="max", **FIRE)
    reps = b.relax(prm)
    X = b.positions()
    for i, a in enumerate(arrs):
        Hi = a["maxy"] - a["miny"]
        x0 = oracle.affine_displace(a["points"], a["miny"], Hi, gam[i] * Hi, 0.0)
        xo, _, _, orep = oracle.Model(a, 1.0, kbs[i]).fire(x0, oracle.params(fcut=1e-10, criterion="max", **FIRE))
        assert reps[i].status == nr.NR_OK
        assert reps[i].steps == orep.steps, i
        assert np.array_equal(X[b.offsets[i]:b.offsets[i + 1]], xo), i
        assert reps[i].e_stretch == orep.e_stretch and reps[i].e_bend == orep.e_bend


def test_sweep_matches_oracle(cuda, fp64_kernel):
    h, a = lattice(16, 0.7, 9)
    net = nr.Network(h, ks=1.0, kb=1e-3)
    prm = nr.fire_params(fcut=1e-10, criterion="max", **FIRE)
    recs, pos = net.sweep([0.01, 0.02, 0.01], [0.01, 0.03, 0.01], prm, keep_positions=True)
    H = a["maxy"] - a["miny"]
    orecs, opos, _ = oracle.Model(a, 1.0, 1e-3).sweep(a["points"], a["miny"], H,
                                                       oracle.params(fcut=1e-10, criterion="max", **FIRE),
                                                       [0.01, 0.02, 0.01], [0.01, 0.03, 0.01])
    assert len(recs) == len(orecs) == 5
    for r, o in zip(recs, orecs):
        assert (r.curr_disp, r.max_comp, r.e_stretch, r.e_bend, r.steps, r.is_shear) == (
            o[0], o[1], o[2], o[3], int(o[6]), int(o[7]))
    shear_rows = [i for i, r in enumerate(recs) if r.is_shear]
    assert np.array_equal(pos[shear_rows], opos[[i for i, o in enumerate(orecs) if o[7] == 1]])


def _rec(r):
    return (r.curr_disp, r.max_comp, r.e_stretch, r.e_bend, r.rms_force, r.max_force, r.steps, r.is_shear,
            r.status)


def test_sweep_graph_equals_step_by_step_sweep(cuda, fp64_kernel):
    """The protocol captured in one CUDA graph gives the step-by-step
    sweep's records and shear positions bit for bit (and so the oracle's:
    test_sweep_matches_oracle)."""
    h, _ = lattice(16, 0.7, 9)
    prm = nr.fire_params(fcut=1e-10, criterion="max", **FIRE)
    compr, shear = [0.01, 0.02, 0.01], [0.01, 0.03, 0.01]
    recs, pos = nr.Network(h, ks=1.0, kb=1e-3).sweep(compr, shear, prm, keep_positions=True, graph=True)
    precs, ppos = nr.Network(h, ks=1.0, kb=1e-3).sweep(compr, shear, prm, keep_positions=True)
    assert len(recs) == len(precs) == 5
    assert [_rec(r) for r in recs] == [_rec(r) for r in precs]
    rows = [i for i, r in enumerate(precs) if r.is_shear]
    assert np.array_equal(pos[rows], ppos[rows])
    # Steps past max_records still run: the final positions agree.
    g, p = nr.Network(h, ks=1.0, kb=1e-3), nr.Network(h, ks=1.0, kb=1e-3)
    r2, _ = g.sweep(compr, shear, prm, max_records=2, graph=True)
    p2, _ = p.sweep(compr, shear, prm, max_records=2)
    assert [_rec(r) for r in r2] == [_rec(r) for r in p2] and len(r2) == 2
    assert np.array_equal(g.positions(), p.positions())


def test_run_fire_md_dropin(cuda, fp64_kernel):
    """The reference's own argument list, device arrays from torch."""
    import torch

    h, a = lattice(24, 0.65, 21)
    N = len(a["points"])
    H = a["maxy"] - a["miny"]
    fc = h.fcodes()
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.02 * H, 0.0)
    dev = cuda
    d_pos = torch.tensor(x0.reshape(-1), dtype=torch.float64, device=dev)
    d_vel = torch.zeros_like(d_pos)
    d_f = torch.zeros_like(d_pos)
    d_pairs = torch.tensor(a["edge_ij"].reshape(-1), dtype=torch.int32, device=dev)
    d_len = torch.tensor(a["edge_l0"], dtype=torch.float64, device=dev)
    d_eoff = torch.tensor(a["edge_wrap"], dtype=torch.int8, device=dev)
    d_tri = torch.tensor(a["tri_hjk"].reshape(-1), dtype=torch.int32, device=dev)
    d_toff = torch.tensor(a["tri_wrap"].reshape(-1), dtype=torch.int8, device=dev)
    d_fc = torch.tensor(fc, dtype=torch.uint8, device=dev)
    fcut = 1e-10 / np.sqrt(2 * N)
    torch.cuda.synchronize()
    st, report, steps = nr.run_fire_md(2 * N, len(a["edge_l0"]), len(a["tri_hjk"]), a["offset"], 1.0, 1e-3,
                                       d_pos.data_ptr(), d_vel.data_ptr(), d_f.data_ptr(), d_pairs.data_ptr(),
                                       d_len.data_ptr(), d_eoff.data_ptr(), d_tri.data_ptr(), d_toff.data_ptr(),
                                       d_fc.data_ptr(), [0.1, 0.99, 0.1, 1.1, 0.5], 1.0, fcut, 10**6, 5)
    xo, vo, Fo, orep = oracle.Model(a, 1.0, 1e-3, fc).fire(x0, oracle.params(fcut=fcut, criterion="rms", **FIRE))
    assert st == nr.NR_OK and steps == orep.steps
    assert np.array_equal(d_pos.cpu().numpy().reshape(-1, 2), xo)
    assert np.array_equal(d_f.cpu().numpy().reshape(-1, 2), Fo)
    assert report == [orep.rms_force, orep.e_stretch, orep.e_bend]


def test_relax_bitwise_mikado(cuda, fp64_kernel):
    """C3-type network (Mikado fibres: per-bond k = 1/l0, per-triple kb and
    rest angles, x-periodic wraps): one shear increment, FP64 relaxation
    identical to the oracle.  dt_max follows the stiffest bond."""
    h = nr.HostNetwork.mikado(300, 0.1, 1.0, 1e-3, 7)
    a = h.arrays()
    prm = dict(FIRE, dt_max=0.1 * float(np.sqrt(a["edge_l0"].min())))
    H = a["maxy"] - a["miny"]
    net = nr.Network(h, ks=1.0, kb=1.0)
    net.affine_displace(a["miny"], H, 0.01 * H, 0.0)
    rep = net.relax(nr.fire_params(fcut=1e-10, criterion="max", **prm))
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.01 * H, 0.0)
    xo, vo, Fo, orep = oracle.Model(a, 1.0, 1.0).fire(x0, oracle.params(fcut=1e-10, criterion="max", **prm))
    assert rep.status == nr.NR_OK and rep.steps == orep.steps
    assert np.array_equal(net.positions(), xo)
    assert rep.e_stretch == orep.e_stretch and rep.e_bend == orep.e_bend


def test_grid_barrier_wait_budget_runs_out_without_a_fault(cuda, monkeypatch):
    """Failure detection without a GPU fault.  NR_TEST_STALL_BARRIER=1 makes
    the FP64 grid kernel's barriers wait for a CTA that was never launched.
    Each wait gives up after its budget (NR_BARRIER_BUDGET_MS), every CTA
    returns, and the relaxation reports NR_ERR_TIMEOUT.  The context stays
    usable: the next relaxation of the same network equals the oracle's."""
    h, a = lattice(12, 0.65, 7)
    H = a["maxy"] - a["miny"]
    net = nr.Network(h, ks=1.0, kb=1e-3)
    net.affine_displace(a["miny"], H, 0.02 * H, 0.0)
    prm = nr.fire_params(fcut=1e-10, criterion="max", **FIRE)
    monkeypatch.setenv("NR_FP64_CLUSTER_NODES", "0")  # the grid kernel, whose barriers are software ones
    monkeypatch.setenv("NR_TEST_STALL_BARRIER", "1")
    monkeypatch.setenv("NR_BARRIER_BUDGET_MS", "20")
    with pytest.raises(nr.NetRelaxError) as e:
        net.relax(prm)
    assert e.value.status == nr.NR_ERR_TIMEOUT
    monkeypatch.delenv("NR_TEST_STALL_BARRIER")
    monkeypatch.delenv("NR_BARRIER_BUDGET_MS")
    rep = net.relax(prm)  # the stalled launch stopped before its first drift: x is the strained start
    x0 = oracle.affine_displace(a["points"], a["miny"], H, 0.02 * H, 0.0)
    x_or, _, _, orep = oracle.Model(a, 1.0, 1e-3).fire(x0, oracle.params(fcut=1e-10, criterion="max", **FIRE))
    assert rep.status == nr.NR_OK and rep.steps == orep.steps
    assert np.array_equal(net.positions(), x_or)


@pytest.mark.parametrize("cache", ["1", "0"])
def test_run_fire_md_dropin_sweep_reuses_image(cuda, cache, monkeypatch):
    """The reference calls run_fire_md once per strain step on the same
    device arrays (large_strain_relax.cu:931, :973).  The drop-in keeps the
    device image it built while the arrays, sizes, constants and contents
    stay the same (a device checksum), and rebuilds it when a value changes
    in place: three warm-started shear steps bit-identical to the oracle's,
    then a rest length changed in place and the next step equal to the
    oracle's on the changed network.  NR_DROPIN_CACHE=0 rebuilds every call:
    the same bits."""
    import torch

    monkeypatch.setenv("NR_DROPIN_CACHE", cache)
    h, a = lattice(20, 0.7, 23)
    N = len(a["points"])
    H = a["maxy"] - a["miny"]
    fc = h.fcodes()
    dev = cuda
    x = a["points"].copy()
    d_pos = torch.tensor(x.reshape(-1), dtype=torch.float64, device=dev)
    d_vel = torch.zeros_like(d_pos)
    d_f = torch.zeros_like(d_pos)
    d_pairs = torch.tensor(a["edge_ij"].reshape(-1), dtype=torch.int32, device=dev)
    d_len = torch.tensor(a["edge_l0"], dtype=torch.float64, device=dev)
    d_eoff = torch.tensor(a["edge_wrap"], dtype=torch.int8, device=dev)
    d_tri = torch.tensor(a["tri_hjk"].reshape(-1), dtype=torch.int32, device=dev)
    d_toff = torch.tensor(a["tri_wrap"].reshape(-1), dtype=torch.int8, device=dev)
    d_fc = torch.tensor(fc, dtype=torch.uint8, device=dev)
    fcut = 1e-10 / np.sqrt(2 * N)
    m = oracle.Model(a, 1.0, 1e-3, fc)

    def step(model):
        nonlocal x
        x = oracle.affine_displace(x, a["miny"], H, 0.01 * H, 0.0)
        d_pos.copy_(torch.tensor(x.reshape(-1), dtype=torch.float64, device=dev))
        torch.cuda.synchronize()
        st, rep, steps = nr.run_fire_md(2 * N, len(a["edge_l0"]), len(a["tri_hjk"]), a["offset"], 1.0, 1e-3,
                                        d_pos.data_ptr(), d_vel.data_ptr(), d_f.data_ptr(), d_pairs.data_ptr(),
                                        d_len.data_ptr(), d_eoff.data_ptr(), d_tri.data_ptr(), d_toff.data_ptr(),
                                        d_fc.data_ptr(), [0.1, 0.99, 0.1, 1.1, 0.5], 1.0, fcut, 10**6, 5)
        xo, _, _, orep = model.fire(x, oracle.params(fcut=fcut, criterion="rms", **FIRE))
        assert st == nr.NR_OK and steps == orep.steps
        assert np.array_equal(d_pos.cpu().numpy().reshape(-1, 2), xo)
        assert rep == [orep.rms_force, orep.e_stretch, orep.e_bend]
        x = xo

    for _ in range(3):
        step(m)
    a2 = dict(a)
    a2["edge_l0"] = a["edge_l0"].copy()
    a2["edge_l0"][5] *= 1.01
    d_len[5] = float(a2["edge_l0"][5])
    step(oracle.Model(a2, 1.0, 1e-3, fc))
