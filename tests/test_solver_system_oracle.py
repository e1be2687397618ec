"""The oracle's restatement of Iron's solver system (Dirichlet elimination) against independent
references: a dense elimination (structure, values, right-hand side to rounding) and a literal
Python transcription of Iron's right-hand-side loop order (bit for bit).  CPU only."""
import numpy as np
import pytest

import oracle
from iron_gb300 import mesh as M

ZERO_TOL = 5.0 * np.finfo(np.float64).eps


def laplace_system(ne, seed):
    m = M.RegularMesh(ne)
    m.jitter_interior(seed)
    kappa = np.exp(np.random.default_rng(seed).uniform(np.log(0.1), np.log(10), m.n_elements))
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    vals, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kappa, rp, ci, 1)
    return m, rp, ci, vals


def dense(rp, ci, vals):
    n = len(rp) - 1
    K = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i] - 1, rp[i + 1] - 1):
            K[i, ci[k] - 1] = vals[k]
    return K


def iron_rhs_loop(rp, ci, vals, f, fixed, u, col_listed):
    """Iron's loop, transcribed: equations rows r ascending; f(r) on free rows; for a fixed r with
    |u(r)| >= tol, -1*K(i,r)*u(r) on every free row i of column r's list with |K(i,r)| >= tol."""
    n = len(rp) - 1
    sod = np.cumsum(~fixed.astype(bool)) - 1
    rows_of_col = [[] for _ in range(n)]
    for i in range(n):
        for k in range(rp[i] - 1, rp[i + 1] - 1):
            c = ci[k] - 1
            if fixed[c] and (col_listed is None or col_listed[c]):
                rows_of_col[c].append((i, vals[k]))
    out = np.zeros(int((~fixed.astype(bool)).sum()))
    for r in range(n):
        if not fixed[r]:
            out[sod[r]] += (0.0 if f is None else f[r]) * 1.0
        if not fixed[r] or not abs(u[r]) >= ZERO_TOL:
            continue
        for i, kv in rows_of_col[r]:
            if fixed[i] or not abs(kv) >= ZERO_TOL:
                continue
            out[sod[i]] += -1.0 * kv * u[r] * 1.0
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_structure_and_values_equal_dense_elimination(seed):
    m, rp, ci, vals = laplace_system((4, 3, 5), seed)
    rng = np.random.default_rng(seed)
    fixed = (rng.uniform(size=m.n_nodes) < 0.3).astype(np.uint8)
    u = rng.standard_normal(m.n_nodes)
    S = oracle.solver_system(rp, ci, vals, None, fixed, u)
    free = np.flatnonzero(fixed == 0)
    assert S["n_free"] == free.size
    np.testing.assert_array_equal(S["solver_of_dof"][free], np.arange(free.size))
    assert (S["solver_of_dof"][fixed == 1] == -1).all()
    K = dense(rp, ci, vals)
    Ks = dense(S["row_ptr"], S["col_idx"], S["values"])
    np.testing.assert_array_equal(Ks, K[np.ix_(free, free)])  # values copied exactly
    # structure: each row's free columns, ascending
    for s_row, r in enumerate(free):
        cols = ci[rp[r] - 1:rp[r + 1] - 1] - 1
        want = S["solver_of_dof"][cols[fixed[cols] == 0]] + 1
        np.testing.assert_array_equal(S["col_idx"][S["row_ptr"][s_row] - 1:S["row_ptr"][s_row + 1] - 1], want)
    # right-hand side: f - K_FD u_D to rounding
    want = -K[np.ix_(free, np.flatnonzero(fixed))] @ u[fixed == 1]
    np.testing.assert_allclose(S["rhs"], want, rtol=0, atol=1e-13 * np.abs(K).max() * np.abs(u).max())


@pytest.mark.parametrize("with_f", [False, True])
def test_rhs_bit_for_bit_with_irons_loop_order(with_f):
    m, rp, ci, vals = laplace_system((3, 4, 3), 2)
    rng = np.random.default_rng(3)
    fixed = (rng.uniform(size=m.n_nodes) < 0.4).astype(np.uint8)
    u = rng.standard_normal(m.n_nodes) * 10.0 ** rng.integers(-17, 3, m.n_nodes)  # some below tolerance
    f = rng.standard_normal(m.n_nodes) if with_f else None
    for col_listed in (None, M.boundary_node_mask((3, 4, 3), 1).astype(np.uint8)):
        S = oracle.solver_system(rp, ci, vals, f, fixed, u, col_listed)
        np.testing.assert_array_equal(S["rhs"], iron_rhs_loop(rp, ci, vals, f, fixed, u, col_listed))


def test_interior_fixed_dof_adds_no_rhs_term_when_lists_hold_boundary_nodes():
    m, rp, ci, vals = laplace_system((3, 3, 3), 4)
    interior = np.flatnonzero(~M.boundary_node_mask((3, 3, 3), 1))
    fixed = np.zeros(m.n_nodes, np.uint8)
    fixed[interior[0]] = 1
    u = np.zeros(m.n_nodes)
    u[interior[0]] = 1.0
    listed = oracle.solver_system(rp, ci, vals, None, fixed, u, M.boundary_node_mask((3, 3, 3), 1).astype(np.uint8))
    every = oracle.solver_system(rp, ci, vals, None, fixed, u, None)
    assert not listed["rhs"].any()
    assert np.count_nonzero(every["rhs"]) == 26  # the fixed node's 26 neighbours
