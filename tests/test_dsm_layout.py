"""The sub-block layout of the thread-block-cluster kernels (batches and
small networks), built and checked on the host (nr_dsm_layout_check):
gather records (each node once, in its own sub-block, ordered by its
numbers of triple and bond entries, ranges and fcode equal to the
incidence lists), item slots owned by the sub-block of the bond's first
node / the triple's hinge, and every resolved incidence entry pointing at
the slot and role it came from."""
import pytest

import network_relaxation_gb300 as nr


@pytest.mark.parametrize("L,p,seed", [(16, 0.65, 1), (48, 0.6, 4), (96, 0.75, 9), (7, 0.9, 2)])
def test_lattice_sub_blocks(built, L, p, seed):
    h = nr.HostNetwork.lattice(L, L, p, 0.0, seed).get_triples()
    st = h.dsm_layout_check()
    assert st["violations"] == 0, st
    assert st["nodes"] == L * L
    assert st["sub_block_nodes"] % 32 == 0 and 1 <= st["sub_blocks"] <= 16


def test_generator_triples_and_per_item_stiffness(built):
    h = nr.HostNetwork.lattice(64, 64, 0.7, 0.05, 3, line_triples=True)
    st = h.dsm_layout_check()
    assert st["violations"] == 0, st


def test_fibre_network_and_reordered_network(built):
    h = nr.HostNetwork.mikado(1200, 0.12, 1.0, 1e-5, 5)
    assert h.dsm_layout_check()["violations"] == 0
    g = nr.HostNetwork.lattice(40, 40, 0.65, 0.0, 6).get_triples()
    g.reorder("morton")
    assert g.dsm_layout_check()["violations"] == 0
