"""Iron's finite-difference Jacobian on the GPU (gfe_mr_jacobian_fd) and the Jacobian-type selector.

Iron's default Jacobian for finite elasticity is one-sided differences of the element residual,
column j = (R(u + delta e_j) - R(u)) / delta with delta = (1 + ||u||_2) * 1e-6
(src/equations_set_routines.F90:2839-2962).  The GPU kernel is compared with the oracle's
restatement of that routine with the same delta: element matrices and assembled CSR values within
1e-9 x max|K| (both sides difference FP64 residuals summed in different orders; the difference
quotient amplifies their rounding by 1/delta).  The Newton known answer (homogeneous uniaxial
stretch) is reached with jacobian="fd", and the selector dispatches to the three Jacobians.
"""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300._lib import GfeError
from iron_gb300.elasticity import MooneyRivlinAssembly
from iron_gb300.newton import NewtonSolver, uniaxial_exact_state, uniaxial_roller_conditions

pytestmark = pytest.mark.gpu

C1, C2 = 2.0, 6.0
STEP = 1e-6


def _state(A, seed, amp=0.02, p=-1.0):
    rng = np.random.default_rng(seed)
    x = A.xg.cpu().numpy()
    lam = 1.05
    z = x * np.array([lam, lam ** -0.5, lam ** -0.5])[:, None]
    z = z + rng.normal(0, amp / A.mesh.nelem[0], z.shape)
    pr = p + rng.normal(0, 0.2, A.n_lin)
    return np.r_[z.ravel(), pr]


def test_element_fd_jacobians_match_oracle(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 1), build_jacobian=False)
    dep = _state(A, 1)
    delta = (1.0 + np.linalg.norm(dep)) * STEP
    K = A.jacobian_fd(torch.from_numpy(dep).cuda(), [C1, C2], step=STEP, dense=True).cpu().numpy()
    x = A.xg.cpu().numpy()
    nq = A.n_q2
    el = A.elin.cpu().numpy()
    for e in range(A.n_elements):
        en = A.mesh.elem_nodes[e]
        Ko = oracle.mr_element_jacobian_fd(x[:, en], dep[: 3 * nq].reshape(3, nq)[:, en], dep[3 * nq:][el[e]], C1, C2,
                                           delta)
        assert np.abs(K[e] - Ko).max() <= 1e-9 * np.abs(Ko).max(), e
        # FD approximates the consistent tangent to O(delta)
    Kt = A.element_tangents(torch.from_numpy(dep).cuda(), [C1, C2]).cpu().numpy()
    assert np.abs(K - Kt).max() <= 1e-3 * np.abs(Kt).max()


@pytest.mark.parametrize("ne", [(1, 1, 1), (3, 2, 2)])
def test_assembled_fd_jacobian_matches_oracle(gfe_cuda, ne):
    A = MooneyRivlinAssembly.from_regular_mesh(ne)
    dep = _state(A, 2)
    delta = (1.0 + np.linalg.norm(dep)) * STEP
    v = A.jacobian_fd(torch.from_numpy(dep).cuda(), [C1, C2], step=STEP).cpu().numpy()
    rp, ci, _ = A.to_iron_csr()
    vo = oracle.mr_assemble_jacobian(A.mesh.elem_nodes, A.elin.cpu().numpy(), A.n_q2, A.n_lin, A.xg.cpu().numpy(),
                                     dep, [C1, C2], rp, ci, fd_delta=delta)
    assert np.abs(v - vo).max() <= 1e-9 * np.abs(vo).max()


def test_jacobian_type_selector(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 2))
    dep = torch.from_numpy(_state(A, 3)).cuda()
    assert A.jacobian_calculation_type == "consistent"
    assert A.jacobian_finite_difference_step_size == 1e-6
    ref = {"consistent": A.tangent(dep, [C1, C2]).clone(), "analytic": A.jacobian(dep, [C1, C2]).clone(),
           "fd": A.jacobian_fd(dep, [C1, C2]).clone()}
    for kind in ("fd", "analytic", "consistent"):
        A.jacobian_calculation_type = kind
        got = A.evaluate_jacobian(dep, [C1, C2])
        assert torch.equal(got, ref[kind]), kind
    A.jacobian_finite_difference_step_size = 1e-7
    A.jacobian_calculation_type = "fd"
    assert not torch.equal(A.evaluate_jacobian(dep, [C1, C2]), ref["fd"])
    with pytest.raises(GfeError):
        A.jacobian_calculation_type = "adjoint-free"
    with pytest.raises(GfeError):
        A.jacobian_finite_difference_step_size = 0.0


def test_newton_uniaxial_stretch_with_fd_jacobian(gfe_cuda):
    lam = 1.1
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 2))
    fixed, full = uniaxial_roller_conditions(A, lam)
    dep = A.initial_state(0.0)
    solver = NewtonSolver(A, [C1, C2], jacobian="fd", absolute_tolerance=1e-12, relative_tolerance=1e-14,
                          solution_tolerance=0.0, linear_relative_tolerance=1e-10)
    assert solver.linear_solver == "gmres"
    infos = solver.solve(dep, fixed, full, load_increments=5)
    assert len(infos) == 5 and all(i.converged for i in infos)
    exact = uniaxial_exact_state(A, lam, C1, C2).cpu().numpy()
    d = dep.cpu().numpy()
    nu = 3 * A.n_q2
    assert np.abs(d[:nu] - exact[:nu]).max() <= 1e-9 * np.abs(exact[:nu]).max()
    assert np.abs(d[nu:] - exact[nu:]).max() <= 1e-8 * abs(exact[nu])
    with pytest.raises(GfeError):
        NewtonSolver(A, [C1, C2], jacobian="fd", linear_solver="minres")
