"""Synthetic workloads of the benchmarks (the reference ships none).

Each builder returns host networks from the seeded generators of the native
library; see nr_gen_lattice in include/netrelax.h.
"""
import numpy as np

from .. import HostNetwork

C4_SEED = 1000
C4_COUNT = 512


def c4_params(n=C4_COUNT, seed=C4_SEED):
    """Per-network parameters of the uneven batch: side L ~ U{16..96},
    bond probability p ~ U[0.55, 0.75], bending stiffness kappa ~
    logU[1e-5, 1e-2], shear strain gamma ~ U[0, 0.1]; network i uses
    generator seed seed + i.  k = 1, triples from get_triples."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.integers(16, 97))
        p = float(rng.uniform(0.55, 0.75))
        kappa = float(10 ** rng.uniform(-5, -2))
        gamma = float(rng.uniform(0, 0.1))
        out.append({"L": L, "p": p, "kappa": kappa, "gamma": gamma, "seed": seed + i})
    return out


def c4_networks(params=None):
    params = params or c4_params()
    return [HostNetwork.lattice(q["L"], q["L"], q["p"], 0.0, q["seed"]).get_triples() for q in params]
