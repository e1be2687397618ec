"""MINRES linear solves and the Newton load-stepping driver on the GPU.

The Newton solve is checked against a known answer: the homogeneous uniaxial stretch of an
incompressible Mooney-Rivlin box with roller conditions, whose exact discrete solution is
z = diag(lam, lam^-1/2, lam^-1/2) x with the uniform traction-free pressure (quadratic u
represents it exactly, and with J = 1 the pressure rows vanish).  Tolerances: state within 1e-10
of max|z| and pressure within 1e-9 of |p|; mixed-precision Newton within 1e-10 of the FP64 result.
The linear solver is checked against a dense LU solve of the same system (scipy/numpy).
"""
import numpy as np
import pytest
import torch

from iron_gb300.elasticity import MooneyRivlinAssembly
from iron_gb300.laplace import LaplaceAssembly
from iron_gb300.mesh import RegularMesh
from iron_gb300.newton import (NewtonSolver, minres_solve, saddle_preconditioner, uniaxial_exact_state,
                               uniaxial_roller_conditions)

pytestmark = pytest.mark.gpu

C1, C2 = 2.0, 6.0


def _dense(rp, ci, v, n):
    A = np.zeros((n, n))
    for r in range(n):
        for k in range(rp[r] - 1, rp[r + 1] - 1):
            A[r, ci[k] - 1] = v[k]
    return A


def _stretched(A, lam, seed):
    dep = uniaxial_exact_state(A, lam, C1, C2).cpu().numpy()
    rng = np.random.default_rng(seed)
    dep[: 3 * A.n_q2] += rng.normal(0, 0.01 / A.mesh.nelem[0], 3 * A.n_q2)
    return torch.from_numpy(dep).cuda()


@pytest.mark.parametrize("nodal", [False, True])
@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-11), ("mixed", 1e-9)])
def test_minres_matches_dense_solve(gfe_cuda, precision, rtol, nodal):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 1))
    dep = _stretched(A, 1.05, 0)
    fixed, _ = uniaxial_roller_conditions(A, 1.05)
    vals = A.tangent(dep, [C1, C2]).clone()
    rng = np.random.default_rng(1)
    f = torch.from_numpy(rng.normal(0, 1, A.ndof)).cuda()
    minv = saddle_preconditioner(A.row_ptr, A.col_idx, vals, 3 * A.n_q2, fixed)
    x = torch.zeros(A.ndof, dtype=torch.float64, device="cuda")
    v32 = vals.float() if precision == "mixed" else None
    info = minres_solve(A.row_ptr, A.col_idx, vals, f, fixed, x, minv=minv, values32=v32, rtol=rtol,
                        precision=precision, n_node=A.n_q2 if nodal else 0)
    assert info.relative_residual <= rtol
    assert info.nodal == (nodal and precision == "mixed")  # FP64 keeps the per-row product
    # dense reference on the free DOFs
    rp, ci, v = A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy(), vals.cpu().numpy()
    K = _dense(rp, ci, v, A.ndof)
    free = fixed.cpu().numpy() == 0
    xr = np.zeros(A.ndof)
    xr[free] = np.linalg.solve(K[np.ix_(free, free)], f.cpu().numpy()[free])
    xg = x.cpu().numpy()
    assert np.abs(xg[~free]).max() == 0.0
    cond_scale = 1e4  # the error of a residual-tolerance solve grows with the condition number
    assert np.abs(xg - xr).max() <= cond_scale * rtol * np.abs(xr).max()


def test_minres_on_spd_system_matches_cg(gfe_cuda):
    m = RegularMesh((6, 5, 4))
    m.jitter_interior(3)
    kap = np.exp(np.random.default_rng(4).uniform(np.log(0.1), np.log(10.0), m.n_elements))
    L = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    L.assemble("fp64")
    fixed = np.zeros(m.n_nodes, np.uint8)
    fixed[m.face_nodes(0, 0)] = 1
    fixed[m.face_nodes(0, 1)] = 1
    x0 = np.where(fixed == 1, m.coords[0], 0.0)
    fixed_t = torch.from_numpy(fixed).cuda()
    x1 = torch.from_numpy(x0).cuda()
    x2 = torch.from_numpy(x0).cuda()
    L.solve(fixed_t, x1, rtol=1e-12)
    info = minres_solve(L.row_ptr, L.col_idx, L.values, None, fixed_t, x2, rtol=1e-13)
    assert info.relative_residual <= 1e-13
    assert (x1 - x2).abs().max().item() <= 1e-10


def test_minres_nodal_product_matches_per_row_product(gfe_cuda):
    """The node-grouped product (u rows of a node share one column list) sums each row in the same
    order as the per-row product; only the inner products add rows in another order, so the two
    solves agree to rounding and take (nearly) the same iterations."""
    A = MooneyRivlinAssembly.from_regular_mesh((4, 3, 3))
    dep = _stretched(A, 1.08, 5)
    fixed, _ = uniaxial_roller_conditions(A, 1.08)
    vals = A.tangent(dep, [C1, C2]).clone()
    f = torch.from_numpy(np.random.default_rng(6).normal(0, 1, A.ndof)).cuda()
    minv = saddle_preconditioner(A.row_ptr, A.col_idx, vals, 3 * A.n_q2, fixed)
    v32 = vals.float()
    rtol = 1e-8
    out = []
    for n_node in (0, A.n_q2):
        x = torch.zeros(A.ndof, dtype=torch.float64, device="cuda")
        info = minres_solve(A.row_ptr, A.col_idx, vals, f, fixed, x, minv=minv, values32=v32, rtol=rtol,
                            precision="mixed", n_node=n_node)
        assert info.relative_residual <= rtol and info.nodal == (n_node > 0)
        out.append((x, info.iterations))
    (x0, i0), (x1, i1) = out
    assert abs(i0 - i1) <= max(2, i0 // 20)
    assert (x0 - x1).abs().max().item() <= 1e3 * rtol * x0.abs().max().item()


def test_minres_nodal_falls_back_when_rows_differ(gfe_cuda):
    """A Laplace matrix read as two components of n/2 nodes: rows i and i + n/2 belong to different
    nodes and hold different column lists, so the solver keeps the per-row product."""
    m = RegularMesh((5, 4, 3))
    L = LaplaceAssembly.from_regular_mesh(m)
    L.assemble("fp64")
    fixed = np.zeros(m.n_nodes, np.uint8)
    fixed[m.face_nodes(0, 0)] = 1
    fixed[m.face_nodes(0, 1)] = 1
    x0 = np.where(fixed == 1, m.coords[0], 0.0)
    fixed_t = torch.from_numpy(fixed).cuda()
    x = torch.from_numpy(x0).cuda()
    v32 = L.values.float()
    info = minres_solve(L.row_ptr, L.col_idx, L.values, None, fixed_t, x, values32=v32, rtol=1e-12,
                        precision="mixed", n_node=m.n_nodes // 2, n_comp=2)
    assert not info.nodal and info.relative_residual <= 1e-12
    assert (x - torch.from_numpy(m.coords[0]).cuda()).abs().max().item() <= 1e-9


def test_saddle_preconditioner_matches_definition(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 1, 1))
    dep = _stretched(A, 1.1, 2)
    fixed, _ = uniaxial_roller_conditions(A, 1.1)
    vals = A.tangent(dep, [C1, C2]).clone()
    minv = saddle_preconditioner(A.row_ptr, A.col_idx, vals, 3 * A.n_q2, fixed).cpu().numpy()
    K = _dense(A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy(), vals.cpu().numpy(), A.ndof)
    nu = 3 * A.n_q2
    fx = fixed.cpu().numpy().astype(bool)
    d = np.abs(np.diag(K))
    mu = np.where(fx[:nu], 0.0, 1.0 / d[:nu])
    S = (K[nu:, :nu] ** 2 * mu[None, :]).sum(1)
    ref = np.r_[mu, np.where(fx[nu:], 0.0, 1.0 / S)]
    assert np.allclose(minv, ref, rtol=1e-13, atol=0)


@pytest.mark.parametrize("ne", [(2, 2, 2), (3, 2, 2)])
def test_newton_uniaxial_stretch_known_answer(gfe_cuda, ne):
    lam = 1.1
    A = MooneyRivlinAssembly.from_regular_mesh(ne)
    fixed, full = uniaxial_roller_conditions(A, lam)
    dep = A.initial_state(0.0)
    solver = NewtonSolver(A, [C1, C2], absolute_tolerance=1e-13, relative_tolerance=1e-14, solution_tolerance=0.0,
                          linear_relative_tolerance=1e-10)
    infos = solver.solve(dep, fixed, full, load_increments=5)
    assert len(infos) == 5 and all(i.converged for i in infos)
    exact = uniaxial_exact_state(A, lam, C1, C2).cpu().numpy()
    d = dep.cpu().numpy()
    nu = 3 * A.n_q2
    assert np.abs(d[:nu] - exact[:nu]).max() <= 1e-10 * np.abs(exact[:nu]).max()
    assert np.abs(d[nu:] - exact[nu:]).max() <= 1e-9 * abs(exact[nu])
    # the consistent tangent gives quadratic convergence: a handful of iterations per load step
    assert max(i.iterations for i in infos) <= 6


def test_newton_mixed_precision_matches_fp64(gfe_cuda):
    lam = 1.1
    A = MooneyRivlinAssembly.from_regular_mesh((3, 3, 2))
    fixed, full = uniaxial_roller_conditions(A, lam)
    # a non-homogeneous problem: a perturbed start and a pulled face with a shear offset
    full = full.clone()
    nq = A.n_q2
    x = A.xg.cpu().numpy()
    onX = torch.from_numpy(np.abs(x[0] - 1.0) < 1e-12).cuda()
    fixed = fixed.clone()
    fixed[nq:2 * nq][onX] = 1
    full[nq:2 * nq][onX] = A.xg[1][onX] + 0.02
    res = {}
    for prec in ("fp64", "mixed"):
        dep = A.initial_state(0.0)
        s = NewtonSolver(A, [C1, C2], precision=prec, absolute_tolerance=1e-13, relative_tolerance=1e-14,
                         solution_tolerance=0.0, linear_relative_tolerance=1e-8)
        s.solve(dep, fixed, full, load_increments=3)
        res[prec] = dep.cpu().numpy()
    assert np.abs(res["mixed"] - res["fp64"]).max() <= 1e-10 * np.abs(res["fp64"]).max()


def test_newton_direction_with_iron_analytic_jacobian(gfe_cuda):
    """Iron's analytic Jacobian (as restated from finite_elasticity_routines.F90) is not the
    derivative of the residual: its u-u block is about 14 % off even in the undeformed state, so a
    full Newton step with it does not reduce the residual (the oracle's dense Newton shows the same),
    while the consistent tangent's step does.  The GPU direction (GMRES on the assembled analytic
    Jacobian) matches the oracle's dense solve of the same system."""
    from iron_gb300.newton import gmres_solve

    lam = 1.05
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 2))
    fixed, full = uniaxial_roller_conditions(A, lam)
    fb = fixed.bool()
    dep = A.initial_state(0.0)
    dep[fb] = full[fb]
    c = [C1, C2]
    R = A.residual(dep, c).clone()
    R[fb] = 0.0
    steps = {}
    for kind in ("analytic", "consistent"):
        vals = (A.jacobian(dep, c) if kind == "analytic" else A.tangent(dep, c)).clone()
        minv = saddle_preconditioner(A.row_ptr, A.col_idx, vals, 3 * A.n_q2, fixed)
        du = torch.zeros_like(dep)
        gmres_solve(A.row_ptr, A.col_idx, vals, -R, fixed, du, minv=minv, rtol=1e-12)
        steps[kind] = du
        if kind == "analytic":
            K = _dense(A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy(), vals.cpu().numpy(), A.ndof)
            free = fixed.cpu().numpy() == 0
            ref = np.zeros(A.ndof)
            ref[free] = np.linalg.solve(K[np.ix_(free, free)], -R.cpu().numpy()[free])
            assert np.abs(du.cpu().numpy() - ref).max() <= 1e-8 * np.abs(ref).max()
    r0 = float(R.norm())
    r_an = A.residual(dep + steps["analytic"], c)
    r_an[fb] = 0.0
    r_co = A.residual(dep + steps["consistent"], c)
    r_co[fb] = 0.0
    assert float(r_co.norm()) < 0.1 * r0
    assert float(r_an.norm()) > r0


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-11), ("mixed", 1e-9)])
def test_gmres_on_iron_analytic_jacobian_matches_dense_solve(gfe_cuda, precision, rtol):
    """Iron's analytic Jacobian is not symmetric; GMRES solves it."""
    from iron_gb300.newton import gmres_solve

    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 1))
    dep = _stretched(A, 1.05, 5)
    fixed, _ = uniaxial_roller_conditions(A, 1.05)
    vals = A.jacobian(dep, [C1, C2]).clone()
    rp, ci, v = A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy(), vals.cpu().numpy()
    K = _dense(rp, ci, v, A.ndof)
    assert np.abs(K - K.T).max() > 1e-8 * np.abs(K).max()
    rng = np.random.default_rng(6)
    f = torch.from_numpy(rng.normal(0, 1, A.ndof)).cuda()
    minv = saddle_preconditioner(A.row_ptr, A.col_idx, vals, 3 * A.n_q2, fixed)
    x = torch.zeros(A.ndof, dtype=torch.float64, device="cuda")
    info = gmres_solve(A.row_ptr, A.col_idx, vals, f, fixed, x, minv=minv,
                       values32=vals.float() if precision == "mixed" else None, rtol=rtol, precision=precision)
    assert info.relative_residual <= rtol
    free = fixed.cpu().numpy() == 0
    xr = np.zeros(A.ndof)
    xr[free] = np.linalg.solve(K[np.ix_(free, free)], f.cpu().numpy()[free])
    xg = x.cpu().numpy()
    assert np.abs(xg[~free]).max() == 0.0
    assert np.abs(xg - xr).max() <= 1e4 * rtol * np.abs(xr).max()
    # the true residual agrees with the reported one
    r = f.cpu().numpy()[free] - K[np.ix_(free, free)] @ xg[free]
    assert np.linalg.norm(r) <= 1.01 * rtol * np.linalg.norm(f.cpu().numpy()[free])


@pytest.mark.parametrize("restart", [5, 30])
def test_gmres_on_spd_system_matches_cg(gfe_cuda, restart):
    from iron_gb300.newton import gmres_solve

    m = RegularMesh((5, 4, 4))
    m.jitter_interior(2)
    L = LaplaceAssembly.from_regular_mesh(m)
    L.assemble("fp64")
    fixed = np.zeros(m.n_nodes, np.uint8)
    fixed[m.face_nodes(0, 0)] = 1
    fixed[m.face_nodes(0, 1)] = 1
    x0 = np.where(fixed == 1, m.coords[0], 0.0)
    fixed_t = torch.from_numpy(fixed).cuda()
    x1 = torch.from_numpy(x0).cuda()
    x2 = torch.from_numpy(x0).cuda()
    L.solve(fixed_t, x1, rtol=1e-12)
    info = gmres_solve(L.row_ptr, L.col_idx, L.values, None, fixed_t, x2, rtol=1e-12, restart=restart)
    assert info.relative_residual <= 1e-12
    assert (x1 - x2).abs().max().item() <= 1e-10
