"""Laplace assembly on higher-order tensor-product Lagrange hexahedra (gfe_laplace_assemble_tp)
and on linear, quadratic and cubic tetrahedra with Gauss_Simplex orders 1..5
against the oracle's restatement of Iron's basis-generic element routine: triquadratic and
tricubic elements, anisotropic Gauss rules, trilinear elements with a non-default rule, FP64 /
float-float / FP32 element arithmetic and the tensor-core (tcgen05 TF32x3) contraction; the patch test u = x on curved (jittered) quadratic and
cubic meshes, through Iron's reduced solve."""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300 import mesh as M
from iron_gb300.laplace import LaplaceAssembly

pytestmark = pytest.mark.gpu


def _problem(ne, order, seed):
    m = M.RegularMesh(ne, order=order)
    m.jitter_interior(seed)
    kap = np.exp(np.random.default_rng(seed).uniform(np.log(0.1), np.log(10.0), m.n_elements))
    return m, kap


@pytest.mark.parametrize("order,n_gauss,ne", [(2, 3, (2, 2, 2)), (3, 4, (2, 1, 2)), (2, (3, 2, 4), (2, 2, 1)),
                                              (1, 3, (3, 2, 2)), (3, 2, (1, 2, 1))])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed_df", 1e-12), ("mixed", 2e-5), ("tf32x3", 2e-5)])
def test_matches_oracle(gfe_cuda, order, n_gauss, ne, precision, tol):
    m, kap = _problem(ne, order, 1)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap, n_gauss=n_gauss)
    assert A.tensor_product
    vals = A.assemble(precision).cpu().numpy()
    rp, ci, _ = A.to_iron_csr()
    orp, oci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    ng = list(n_gauss) if np.ndim(n_gauss) else [n_gauss] * 3
    ref, _ = oracle.laplace_assemble(3, [order] * 3, ng, m.elem_nodes, m.coords, kap, orp, oci, 1)
    assert np.abs(vals - ref).max() <= tol * np.abs(ref).max()
    if precision != "fp64":
        assert A.values32 is not None
        assert np.array_equal(A.values32.cpu().numpy(), vals.astype(np.float32))


@pytest.mark.parametrize("order,n_gauss", [(2, 3), (3, 4), (3, 2)])
@pytest.mark.parametrize("precision", ["fp64", "mixed_df", "tf32x3"])
def test_slot_map_equals_search(gfe_cuda, order, n_gauss, precision):
    """The element slot map holds the positions Iron's row search finds: assembling through it gives
    bit-identical values to searching every entry during the assembly."""
    m, kap = _problem((2, 3, 2), order, 3)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap, n_gauss=n_gauss, slot_map=True)
    B = LaplaceAssembly.from_regular_mesh(m, kappa=kap, n_gauss=n_gauss, slot_map=False)
    va = A.assemble(precision).clone()
    vb = B.assemble(precision)
    assert A.tp_slots is not None and B.tp_slots is None
    assert int((A.tp_slots < 0).sum()) == 0
    assert torch.equal(va, vb)


@pytest.mark.parametrize("order", [2, 3])
def test_patch_test_through_reduced_solve(gfe_cuda, order):
    """u = x is reproduced on interior-jittered (curved) quadratic elements, where 3-point Gauss
    integrates the metric terms exactly, and on axis-stretched (affine) cubic elements; on curved
    cubic elements the integrand exceeds what 4-point Gauss integrates exactly.  (The lateral faces
    must stay normal to y and z, or u = x would violate their zero-flux condition.)"""
    m = M.RegularMesh((3, 2, 2), order=order)
    if order == 2:
        m.jitter_interior(4)
    else:
        m.coords = m.coords * np.array([1.0, 0.7, 1.6])[:, None]
    A = LaplaceAssembly.from_regular_mesh(m)  # unit conductivity
    A.assemble("fp64")
    fixed = torch.zeros(m.n_nodes, dtype=torch.uint8, device="cuda")
    x = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
    right = torch.from_numpy(m.face_nodes(0, 1)).cuda()
    fixed[torch.from_numpy(m.face_nodes(0, 0)).cuda()] = 1
    fixed[right] = 1
    x[right] = 1.0
    info = A.solve_reduced(fixed, x, rtol=1e-13)
    assert info.relative_residual <= 1e-13
    assert (x - torch.from_numpy(m.coords[0]).cuda()).abs().max().item() <= 1e-10


def test_rejects_unsupported_bases(gfe_cuda):
    m = M.RegularMesh((1, 1, 1), order=2)
    with pytest.raises(Exception, match="Gauss"):
        LaplaceAssembly.from_regular_mesh(m, n_gauss=5).assemble("fp64")
    # the tensor-core contraction covers hexahedral bases only
    tm = M.TetMesh((1, 1, 1), order=2)
    with pytest.raises(Exception, match="hexahedral"):
        LaplaceAssembly.from_tet_mesh(tm).assemble("tf32x3")


@pytest.mark.parametrize("scaling", ["unit", "arc_length"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed_df", 1e-12), ("mixed", 2e-5), ("tf32x3", 2e-5)])
def test_cubic_hermite_matches_oracle(gfe_cuda, scaling, precision, tol):
    hm = M.HermiteMesh((2, 2, 2), extent=(1.0, 0.8, 1.2), scaling=scaling)
    hm.jitter_interior(5)
    kap = np.exp(np.random.default_rng(6).uniform(np.log(0.1), np.log(10.0), hm.n_elements))
    A = LaplaceAssembly.from_hermite_mesh(hm, kappa=kap)
    vals = A.assemble(precision).cpu().numpy()
    rp, ci, _ = A.to_iron_csr()
    orp, oci = oracle.csr_structure(hm.elem_params, hm.n_dofs)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    ref = oracle.laplace_assemble_scaled(3, [4, 4, 4], [4, 4, 4], hm.elem_params, hm.params, hm.scale, kap, orp, oci)
    assert np.abs(vals - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("scaling", ["unit", "arc_length"])
def test_cubic_hermite_patch_test(gfe_cuda, scaling):
    """u = x on a stretched box: every parameter of the x = 0 and x = 1 face nodes fixed to the
    exact parameters (value x, d/ds1 of x, zero elsewhere); the reduced solve returns the exact
    parameters at every other DOF."""
    hm = M.HermiteMesh((3, 2, 2), extent=(1.0, 0.7, 1.4), scaling=scaling)
    A = LaplaceAssembly.from_hermite_mesh(hm)
    A.assemble("fp64")
    exact = torch.from_numpy(hm.params[0].copy()).cuda()
    fixed = torch.zeros(hm.n_dofs, dtype=torch.uint8, device="cuda")
    for side in (0, 1):
        fixed[torch.from_numpy(hm.face_dofs(0, side)).cuda()] = 1
    x = torch.where(fixed.bool(), exact, torch.zeros_like(exact))
    info = A.solve_reduced(fixed, x, rtol=1e-13, system=A.solver_system(fixed, col_listed=None))
    assert info.relative_residual <= 1e-13
    assert (x - exact).abs().max().item() <= 1e-10


@pytest.mark.parametrize("order,quad", [(1, 1), (1, 2), (1, 5), (2, 2), (2, 3), (2, 4), (3, 3), (3, 4), (3, 5)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed_df", 1e-12), ("mixed", 2e-5)])
def test_tetrahedra_match_oracle(gfe_cuda, order, quad, precision, tol):
    tm = M.TetMesh((3, 2, 2), order=order, extent=(1.0, 0.8, 1.2))
    tm.jitter_interior(7)
    kap = np.exp(np.random.default_rng(8).uniform(np.log(0.1), np.log(10.0), tm.n_elements))
    A = LaplaceAssembly.from_tet_mesh(tm, kappa=kap, n_gauss=quad)
    vals = A.assemble(precision).cpu().numpy()
    rp, ci, _ = A.to_iron_csr()
    orp, oci = oracle.csr_structure(tm.elem_nodes, tm.n_nodes)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    ref = oracle.laplace_assemble_scaled(3, [6 + order] * 3, [quad] * 3, tm.elem_nodes, tm.coords, None, kap, orp, oci)
    assert np.abs(vals - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("order", [1, 2, 3])
def test_tetrahedra_patch_test(gfe_cuda, order):
    tm = M.TetMesh((3, 3, 2), order=order)
    tm.jitter_interior(9)
    A = LaplaceAssembly.from_tet_mesh(tm)
    A.assemble("fp64")
    fixed = torch.zeros(tm.n_nodes, dtype=torch.uint8, device="cuda")
    x = torch.zeros(tm.n_nodes, dtype=torch.float64, device="cuda")
    right = torch.from_numpy(tm.face_nodes(0, 1)).cuda()
    fixed[torch.from_numpy(tm.face_nodes(0, 0)).cuda()] = 1
    fixed[right] = 1
    x[right] = 1.0
    info = A.solve_reduced(fixed, x, rtol=1e-13, system=A.solver_system(fixed, col_listed=None))
    assert info.relative_residual <= 1e-13
    assert (x - torch.from_numpy(tm.coords[0]).cuda()).abs().max().item() <= 1e-10
