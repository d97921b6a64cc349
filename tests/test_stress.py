"""Stress outputs (no counterpart in the reference, which reports energies
only): the virial W = -sum_n r_n (x) F_n of the stretch and bending forces,
sigma = W / A.  Checked here on the oracle (CPU):

* W is the derivative of the energy under the homogeneous deformations the
  protocol applies: W_xy = dE/dgamma under affine_displace's shear
  (large_strain_relax.cu:527-537), W_yy under the y stretch, W_xx under an x
  stretch with the period scaled too -- central finite differences at a
  fixed configuration;
* at a relaxed state sigma_xy = (1/A) dE*/dgamma for the RELAXED energy
  E*(gamma) of the shear protocol (the clamped rows carry the load), by
  finite differences of relaxations at gamma +- h;
* per-item terms reduced with the canonical tree: the total equals the
  plain sum of the items to rounding."""
import numpy as np

import network_relaxation_gb300 as nr
import oracle


def _lattice(L, p, seed, jitter=0.0):
    if jitter > 0:
        h = nr.HostNetwork.lattice(L, L, p, jitter, seed, line_triples=True)
    else:
        h = nr.HostNetwork.lattice(L, L, p, 0.0, seed).get_triples()
    return h.arrays()


def _deformed(a, x, kind, eps):
    y0 = a["miny"]
    out = np.array(x, dtype=np.float64, copy=True)
    if kind == "xy":
        out[:, 0] += eps * (x[:, 1] - y0)
    elif kind == "yy":
        out[:, 1] += eps * (x[:, 1] - y0)
    else:  # xx
        out[:, 0] *= 1.0 + eps
    return out


def _model(a, ks, kb, width=None):
    b = dict(a)
    if width is not None:
        b["offset"] = width
    return oracle.Model(b, ks, kb)


def test_virial_is_the_affine_derivative_of_the_energy():
    a = _lattice(14, 0.8, 3, jitter=0.05)
    rng = np.random.default_rng(1)
    x = a["points"] + rng.normal(0.0, 0.02, a["points"].shape)  # a generic, unrelaxed state
    ks, kb = 1.0, 3e-2
    m = _model(a, ks, kb)
    W = m.virial(x)
    h = 1e-6
    for c, kind in enumerate(("xx", "yy", "xy")):
        if kind == "xx":
            ep = sum(_model(a, ks, kb, a["offset"] * (1 + h)).energies(_deformed(a, x, kind, h)))
            em = sum(_model(a, ks, kb, a["offset"] * (1 - h)).energies(_deformed(a, x, kind, -h)))
        else:
            ep = sum(m.energies(_deformed(a, x, kind, h)))
            em = sum(m.energies(_deformed(a, x, kind, -h)))
        fd = (ep - em) / (2 * h)
        assert abs(fd - W[c]) <= 1e-6 * max(abs(W[c]), 1e-3), (kind, fd, W[c])


def test_virial_total_is_the_canonical_sum_of_item_terms():
    a = _lattice(10, 0.75, 4)
    x = a["points"] + np.random.default_rng(2).normal(0.0, 0.01, a["points"].shape)
    W = _model(a, 1.0, 1e-2).virial(x)
    Wb = _model(a, 1.0, 0.0).virial(x)  # bonds only
    Wt = _model(a, 0.0, 1e-2).virial(x)  # triples only
    assert np.array_equal(W, Wb + Wt)
    # bonds: central forces, so W_xy of the bonds alone equals sum r_x f_y too
    ij, w = a["edge_ij"], a["edge_wrap"].astype(np.float64)
    r = x[ij[:, 1]] + np.column_stack([w * a["offset"], np.zeros_like(w)]) - x[ij[:, 0]]
    lr = np.sqrt((r ** 2).sum(1))
    f = (1.0 - a["edge_l0"] / lr)[:, None] * r  # force on i
    assert np.allclose(Wb, [np.sum(r[:, 0] * f[:, 0]), np.sum(r[:, 1] * f[:, 1]), np.sum(r[:, 1] * f[:, 0])],
                       rtol=1e-12, atol=1e-15)
    assert abs(np.sum(r[:, 0] * f[:, 1]) - Wb[2]) <= 1e-12 * abs(Wb[2]) + 1e-15


def test_relaxed_shear_stress_is_the_derivative_of_the_relaxed_energy():
    """sigma_xy(gamma) = (1/A) dE*/dgamma along the shear protocol."""
    a = _lattice(12, 0.85, 7)
    ks, kb = 1.0, 1e-2
    m = _model(a, ks, kb)
    H = a["maxy"] - a["miny"]
    A = a["offset"] * H
    prm = oracle.params(fcut=1e-13, criterion="max", max_steps=10**6)
    gam, h = 0.04, 2e-4
    x0 = oracle.affine_displace(a["points"], a["miny"], H, gam * H, 0.0)
    xr, _, _, rep = m.fire(x0, prm)
    assert rep.converged
    sigma = m.virial(xr)[2] / A
    e = {}
    for s in (-1, 1):
        xs = oracle.affine_displace(xr, a["miny"], H, s * h * H, 0.0)
        xs, _, _, r2 = m.fire(xs, prm)
        assert r2.converged
        e[s] = sum(m.energies(xs))
    fd = (e[1] - e[-1]) / (2 * h) / A
    assert abs(fd - sigma) <= 1e-5 * abs(sigma), (fd, sigma)
    # the secant modulus from the energy and the stress agree at small strain
    assert sigma > 0
