"""Known answers for the oracle's tetrahedral bases and Gauss_Simplex rules (CPU only): on the unit
tetrahedron the element matrix annihilates constants for every rule, and u^T K u equals the exact
Dirichlet energy of a polynomial the basis reproduces whenever the rule integrates |grad u|^2
exactly -- x (linear), x^2 (quadratic: 1/15), x^3 (cubic: 3/70), with Iron's node orders
(src/basis_routines.F90:4813-5875) and rules of orders 1..5 (:6898-7600)."""
import numpy as np
import pytest

import oracle
from iron_gb300.mesh import CUBIC_TET_POSITIONS

VERTS = np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]])
QUAD_POSITIONS = [(3, 1, 1, 1), (1, 3, 1, 1), (1, 1, 3, 1), (1, 1, 1, 3), (2, 2, 1, 1), (2, 1, 2, 1), (2, 1, 1, 2),
                  (1, 2, 2, 1), (1, 1, 2, 2), (1, 2, 1, 2)]
LIN_POSITIONS = [(2, 1, 1, 1), (1, 2, 1, 1), (1, 1, 2, 1), (1, 1, 1, 2)]


def _nodes(p):
    pos = {1: LIN_POSITIONS, 2: QUAD_POSITIONS, 3: CUBIC_TET_POSITIONS}[p]
    w = (np.array(pos, dtype=float) - 1.0) / p  # area coordinates of the nodes
    return VERTS @ w.T  # [3][nns]


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("rule", [1, 2, 3, 4, 5])
def test_element_annihilates_constants(p, rule):
    K = oracle.laplace_element(3, [6 + p] * 3, [rule] * 3, _nodes(p))
    assert np.abs(K @ np.ones(K.shape[0])).max() <= 1e-12 * np.abs(K).max()
    assert np.allclose(K, K.T, rtol=0, atol=1e-14 * np.abs(K).max())


@pytest.mark.parametrize("p,exact_from", [(1, 1), (2, 2), (3, 4)])
@pytest.mark.parametrize("rule", [1, 2, 3, 4, 5])
def test_energy_of_reproduced_polynomial(p, exact_from, rule):
    x = _nodes(p)
    K = oracle.laplace_element(3, [6 + p] * 3, [rule] * 3, x)
    u = x[0] ** p
    energy = {1: 1.0 / 6.0, 2: 1.0 / 15.0, 3: 3.0 / 70.0}[p]  # integral of |d(x^p)/dx|^2
    got = u @ K @ u
    if rule >= exact_from:
        assert abs(got - energy) <= 1e-13 * energy, (got, energy)
    else:
        assert abs(got - energy) > 1e-10 * energy  # an inexact rule shows


def test_rule_weights_sum_to_volume():
    for rule in (1, 2, 3, 4, 5):
        # constant conductivity, u = x: energy = volume for every rule (the gradient is constant)
        K = oracle.laplace_element(3, [7] * 3, [rule] * 3, VERTS)
        u = VERTS[0]
        assert abs(u @ K @ u - 1.0 / 6.0) <= 1e-15
