"""The spatial tile layout of the tiled mixed-precision kernel, built and
checked on the host (nr_tile_layout_check): every node owned by exactly one
tile, every local reference, incidence entry and halo position inside its
tile, bond entries before triple entries per node, 16-byte aligned records,
fcodes copied; equal-count cells give a tile count that is a multiple of
the CTA count and records of similar size even on fibre networks."""
import pytest

import network_relaxation_gb300 as nr


@pytest.mark.parametrize("side,ctas,target", [(256, 152, 512), (200, 304, 256), (96, 152, 64), (300, 152, 512)])
def test_lattice_layout(built, side, ctas, target):
    h = nr.HostNetwork.lattice(side, side, 0.65, 0.05, 5, line_triples=True)
    st = h.tile_layout_check(ctas, target)
    assert st["violations"] == 0, st
    n = side * side
    per = ctas * target
    assert st["tiles"] == ctas * ((n + per - 1) // per)  # equal-count cells: exactly the planned count
    assert st["positions"] >= n and st["positions"] % 16 == 0
    assert st["max_record_bytes"] % 16 == 0
    # a spatial tile's halo is a thin rim: well under its own node count
    assert st["halo_nodes"] < 0.8 * n


def test_lattice_with_get_triples_and_dilution(built):
    h = nr.HostNetwork.lattice(150, 150, 0.55, 0.0, 9).get_triples()
    st = h.tile_layout_check(152, 128)
    assert st["violations"] == 0, st


def test_fibre_network_layout_is_balanced(built):
    """Mikado networks are spread unevenly in space; equal-count cells keep
    the largest tile record near the mean (uniform cells would double it)."""
    h = nr.HostNetwork.mikado(4000, 0.08, 1.0, 1e-5, 3)
    st = h.tile_layout_check(152, 256)
    assert st["violations"] == 0, st
    assert st["tiles"] % 152 == 0
    n_tiles = st["tiles"]
    mean_nodes = h.n_points / n_tiles
    assert st["max_tile_nodes"] < 4 * mean_nodes


def test_tiny_network_and_errors(built):
    h = nr.HostNetwork.lattice(8, 8, 0.65, 0.0, 1).get_triples()
    st = h.tile_layout_check(152, 512)  # fewer nodes than cells: empty cells are dropped
    assert st["violations"] == 0 and 0 < st["tiles"] <= 64
    with pytest.raises(nr.NetRelaxError):
        h.tile_layout_check(0, 512)
