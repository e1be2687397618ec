"""Host-side mesh generation is Iron-identical (checked against the oracle) and the colourings
are valid (CPU only)."""
import numpy as np
import pytest

import oracle
from iron_gb300 import mesh as M


@pytest.mark.parametrize("ne", [(1, 1, 1), (2, 3, 4), (5, 1, 2), (8, 8, 8)])
@pytest.mark.parametrize("order", [1, 2])
def test_regular_mesh_matches_oracle(ne, order):
    assert np.array_equal(M.regular_elements(ne, order), oracle.regular_mesh(ne, order))
    a = M.regular_coords(ne, order, (0.5, -1.0, 2.0), (1.0, 2.0, 3.0))
    b = oracle.regular_coords(ne, order, (0.5, -1.0, 2.0), (1.0, 2.0, 3.0))
    assert np.array_equal(a, b)


def test_linear_component_matches_oracle():
    e2 = M.regular_elements((3, 2, 2), 2)
    el, g = M.linear_component(e2, 2)
    el2, g2 = oracle.linear_component(e2, (3, 3, 3))
    assert np.array_equal(el, el2) and np.array_equal(g, g2)
    assert len(g) == 4 * 3 * 3


def _check_colouring(elem_nodes, order, ptr):
    assert ptr[0] == 0 and ptr[-1] == elem_nodes.shape[0]
    assert np.array_equal(np.sort(order), np.arange(elem_nodes.shape[0]))
    for c in range(len(ptr) - 1):
        nodes = elem_nodes[order[ptr[c]:ptr[c + 1]]].reshape(-1)
        assert len(np.unique(nodes)) == len(nodes), f"colour {c} shares a node"


@pytest.mark.parametrize("ne", [(1, 1, 1), (3, 3, 3), (4, 2, 5)])
def test_parity_colouring_valid(ne):
    m = M.RegularMesh(ne)
    order, ptr = m.colouring()
    _check_colouring(m.elem_nodes, order, ptr)


def test_greedy_colouring_valid_on_permuted_mesh():
    m = M.RegularMesh((4, 3, 3))
    rng = np.random.default_rng(3)
    perm = rng.permutation(m.n_elements)
    en = m.elem_nodes[perm]
    order, ptr = M.greedy_colouring(en, m.n_nodes)
    _check_colouring(en, order, ptr)
    assert len(ptr) - 1 <= 27


def test_jitter_keeps_boundary_and_is_seeded():
    a = M.RegularMesh((4, 4, 4)); a.jitter_interior(7)
    b = M.RegularMesh((4, 4, 4)); b.jitter_interior(7)
    c = M.RegularMesh((4, 4, 4))
    assert np.array_equal(a.coords, b.coords)
    bnd = M.boundary_node_mask((4, 4, 4), 1)
    assert np.array_equal(a.coords[:, bnd], c.coords[:, bnd])
    d = np.abs(a.coords - c.coords)[:, ~bnd]
    assert d.max() <= 0.1 * 0.25 + 1e-15 and d.max() > 0.01
