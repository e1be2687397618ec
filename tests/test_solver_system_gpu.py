"""Iron's solver system on the GPU (csrc/dirichlet.cu) against the oracle's restatement: the
reduced CSR structure, the values and the right-hand side are bit-identical for Laplace systems
(Dirichlet faces, random fixed sets with interior DOFs and values below Iron's zero tolerance,
with and without an equations right-hand side, with Iron's boundary-node column lists and with
every column listed) and for the non-symmetric Mooney-Rivlin Jacobian (rows of up to 375 entries);
the reduced solve reproduces the full-space solve and the patch test."""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300 import mesh as M
from iron_gb300.elasticity import MooneyRivlinAssembly
from iron_gb300.laplace import LaplaceAssembly
from iron_gb300.solver_system import SolverSystem

pytestmark = pytest.mark.gpu


def _laplace(ne, seed):
    m = M.RegularMesh(ne)
    m.jitter_interior(seed)
    kap = np.exp(np.random.default_rng(seed).uniform(np.log(0.1), np.log(10.0), m.n_elements))
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    A.assemble("fp64")
    return m, A


def _compare(S, values, u, f, fixed, col_listed):
    rp, ci = S.eq_row_ptr.cpu().numpy(), S.eq_col_idx.cpu().numpy()
    O = oracle.solver_system(rp, ci, values.cpu().numpy(), None if f is None else f.cpu().numpy(), fixed, u.cpu().numpy(),
                             col_listed)
    assert S.n_free == O["n_free"] and S.nnz == len(O["col_idx"])
    np.testing.assert_array_equal(S.solver_of_dof.cpu().numpy(), O["solver_of_dof"])
    np.testing.assert_array_equal(S.row_ptr.cpu().numpy(), O["row_ptr"])
    np.testing.assert_array_equal(S.col_idx.cpu().numpy(), O["col_idx"])
    v, v32 = S.matrix(values, fp32=True)
    np.testing.assert_array_equal(v.cpu().numpy(), O["values"])
    np.testing.assert_array_equal(v32.cpu().numpy(), O["values"].astype(np.float32))
    np.testing.assert_array_equal(S.rhs(values, u, f).cpu().numpy(), O["rhs"])


@pytest.mark.parametrize("case", ["faces", "random", "random_f"])
def test_laplace_solver_system_bit_identical_to_oracle(gfe_cuda, case):
    m, A = _laplace((8, 8, 8), 0)
    n = m.n_nodes
    rng = np.random.default_rng(7)
    if case == "faces":
        fixed = np.zeros(n, np.uint8)
        fixed[m.face_nodes(0, 0)] = 1
        fixed[m.face_nodes(0, 1)] = 1
        u = np.zeros(n)
        u[m.face_nodes(0, 1)] = 1.0
    else:
        fixed = (rng.uniform(size=n) < 0.3).astype(np.uint8)
        u = rng.standard_normal(n) * 10.0 ** rng.integers(-17, 2, n)
    f = torch.from_numpy(rng.standard_normal(n)).cuda() if case == "random_f" else None
    ut = torch.from_numpy(u).cuda()
    boundary = M.boundary_node_mask((8, 8, 8), 1).astype(np.uint8)
    for col_listed in (boundary, None):
        S = SolverSystem(A.row_ptr, A.col_idx, torch.from_numpy(fixed).cuda(),
                         None if col_listed is None else torch.from_numpy(col_listed).cuda())
        _compare(S, A.values, ut, f, fixed, col_listed)
    S = A.solver_system(torch.from_numpy(fixed).cuda())  # boundary-node lists by default
    _compare(S, A.values, ut, f, fixed, boundary)


def test_mr_jacobian_solver_system_bit_identical_to_oracle(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((3, 2, 2))
    rng = np.random.default_rng(5)
    x = A.xg.cpu().numpy()
    dep = np.r_[(x * np.array([1.05, 1.05 ** -0.5, 1.05 ** -0.5])[:, None]).ravel(), -1.0 + rng.normal(0, 0.1, A.n_lin)]
    vals = A.jacobian(torch.from_numpy(dep).cuda(), [2.0, 6.0]).clone()
    fixed = (rng.uniform(size=A.ndof) < 0.2).astype(np.uint8)
    u = torch.from_numpy(rng.standard_normal(A.ndof)).cuda()
    S = SolverSystem(A.row_ptr, A.col_idx, torch.from_numpy(fixed).cuda())
    assert int((S.eq_row_ptr[1:] - S.eq_row_ptr[:-1]).max()) > 64  # rows span several warp chunks
    _compare(S, vals, u, None, fixed, None)


def test_all_fixed_and_none_fixed(gfe_cuda):
    m, A = _laplace((2, 2, 2), 1)
    n = m.n_nodes
    S = A.solver_system(torch.ones(n, dtype=torch.uint8, device="cuda"), col_listed=None)
    assert S.n_free == 0 and S.nnz == 0
    assert S.matrix(A.values).numel() == 0 and S.rhs(A.values, torch.zeros(n, dtype=torch.float64, device="cuda")).numel() == 0
    S = A.solver_system(torch.zeros(n, dtype=torch.uint8, device="cuda"), col_listed=None)
    assert S.n_free == n and S.nnz == A.nnz
    assert torch.equal(S.col_idx, A.col_idx) and torch.equal(S.matrix(A.values), A.values)


@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_reduced_solve_matches_full_space_solve_and_patch_test(gfe_cuda, precision):
    m = M.RegularMesh((8, 8, 8))
    m.jitter_interior(3)
    A = LaplaceAssembly.from_regular_mesh(m)  # unit conductivity: the patch test u = x holds
    A.assemble(precision, fp32_copy=precision != "fp64")
    fixed = torch.zeros(m.n_nodes, dtype=torch.uint8, device="cuda")
    x0 = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
    left, right = torch.from_numpy(m.face_nodes(0, 0)).cuda(), torch.from_numpy(m.face_nodes(0, 1)).cuda()
    fixed[left] = 1
    fixed[right] = 1
    x0[right] = 1.0
    xr, xf = x0.clone(), x0.clone()
    ir = A.solve_reduced(fixed, xr, rtol=1e-12, precision=precision)
    if_ = A.solve(fixed, xf, rtol=1e-12, precision=precision)
    assert ir.relative_residual <= 1e-12 and if_.relative_residual <= 1e-12
    assert (xr - xf).abs().max().item() <= 1e-10
    exact = torch.from_numpy(m.coords[0]).cuda()
    assert (xr - exact).abs().max().item() <= 1e-10
    assert torch.equal(xr[fixed.bool()], x0[fixed.bool()])
