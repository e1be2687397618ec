"""Iron's own Python example sequences run against the Iron-shaped surface on the GPU.

- bindings/python/tests/Laplace.py:99-187 (trilinear Laplace on a 5x5x5 regular generated mesh of
  extent 2 x 1 x 3, u = 0 at the first node and u = 1 at the last, iterative solve to 1e-12): the
  nodal solution matches the oracle's (Iron's element loop restated in C++, with its own CG) within
  1e-9 relative, and the equations matrix read back with LinearMatrixGet / StorageLocationsGet /
  DataGet has Iron's CSR structure (bit-identical) and the oracle's values within 1e-13 x max|K|;
- the same sequence with the generalised Laplace subtype: isotropic element conductivities in
  the materials field's three diagonal components (the standard element loop), and a full
  anisotropic tensor with a three-angle nodal fibre field as Iron's geometric-fibre field (the
  generalised element loop and GMRES), matching the oracle's generalised assembly within
  1e-13 x max|K| and a direct solve of the oracle's system within 1e-9;
- the Mooney-Rivlin sequence of bindings/python/tests/Cantilever.py restricted to the covered
  elements (triquadratic displacement, trilinear node-based pressure basis, no body force): a
  homogeneous uniaxial stretch with roller conditions set by AddNode / SetNode, solved in load
  increments with Iron's default finite-difference Jacobian and with the analytic-Jacobian
  selector, reaching the exact state within 1e-9;
- the context's mesh cache: a second mesh handle of the same connectivity reuses the structure.
"""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300 import iron
from iron_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _laplace_sequence(subtype=iron.EquationsSetSubtypes.STANDARD_LAPLACE, cond=None, n=5, fibre=None):
    height, width, length = 1.0, 2.0, 3.0
    coordinateSystem = iron.CoordinateSystem()
    coordinateSystem.CreateStart(1)
    coordinateSystem.dimension = 3
    coordinateSystem.CreateFinish()
    region = iron.Region()
    region.CreateStart(2, iron.WorldRegion)
    region.label = "LaplaceRegion"
    region.coordinateSystem = coordinateSystem
    region.CreateFinish()
    basis = iron.Basis()
    basis.CreateStart(3)
    basis.type = iron.BasisTypes.LAGRANGE_HERMITE_TP
    basis.numberOfXi = 3
    basis.interpolationXi = [iron.BasisInterpolationSpecifications.LINEAR_LAGRANGE] * 3
    basis.quadratureNumberOfGaussXi = [2] * 3
    basis.CreateFinish()
    generatedMesh = iron.GeneratedMesh()
    generatedMesh.CreateStart(4, region)
    generatedMesh.type = iron.GeneratedMeshTypes.REGULAR
    generatedMesh.basis = [basis]
    generatedMesh.extent = [width, height, length]
    generatedMesh.numberOfElements = [n, n, n]
    mesh = iron.Mesh()
    generatedMesh.CreateFinish(5, mesh)
    decomposition = iron.Decomposition()
    decomposition.CreateStart(6, mesh)
    decomposition.type = iron.DecompositionTypes.CALCULATED
    decomposition.numberOfDomains = iron.ComputationalNumberOfNodesGet()
    decomposition.CreateFinish()
    geometricField = iron.Field()
    geometricField.CreateStart(7, region)
    geometricField.meshDecomposition = decomposition
    for c in (1, 2, 3):
        geometricField.ComponentMeshComponentSet(iron.FieldVariableTypes.U, c, 1)
    geometricField.CreateFinish()
    generatedMesh.GeometricParametersCalculate(geometricField)
    geometricFibreField = geometricField
    if fibre is not None:
        fibreField = iron.Field()
        fibreField.CreateStart(13, region)
        fibreField.TypeSet(iron.FieldTypes.FIBRE)
        fibreField.MeshDecompositionSet(decomposition)
        fibreField.GeometricFieldSet(geometricField)
        fibreField.NumberOfComponentsSet(iron.FieldVariableTypes.U, fibre.shape[0])
        fibreField.CreateFinish()
        for c in range(fibre.shape[0]):
            for k in range(fibre.shape[1]):
                fibreField.ParameterSetUpdateNodeDP(iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES,
                                                    1, 1, k + 1, c + 1, float(fibre[c, k]))
        geometricFibreField = fibreField
    equationsSetField = iron.Field()
    equationsSet = iron.EquationsSet()
    spec = [iron.EquationsSetClasses.CLASSICAL_FIELD, iron.EquationsSetTypes.LAPLACE_EQUATION, subtype]
    equationsSet.CreateStart(10, region, geometricFibreField, spec, 8, equationsSetField)
    equationsSet.CreateFinish()
    dependentField = iron.Field()
    equationsSet.DependentCreateStart(9, dependentField)
    dependentField.DOFOrderTypeSet(iron.FieldVariableTypes.U, iron.FieldDOFOrderTypes.SEPARATED)
    dependentField.DOFOrderTypeSet(iron.FieldVariableTypes.DELUDELN, iron.FieldDOFOrderTypes.SEPARATED)
    equationsSet.DependentCreateFinish()
    dependentField.ComponentValuesInitialiseDP(iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES, 1, 0.5)
    if cond is not None:
        materialsField = iron.Field()
        equationsSet.MaterialsCreateStart(11, materialsField)
        equationsSet.MaterialsCreateFinish()
        for c in range(6):
            for e, k in enumerate(cond[c]):
                materialsField.ParameterSetUpdateElementDP(iron.FieldVariableTypes.U,
                                                           iron.FieldParameterSetTypes.VALUES, e + 1, c + 1, float(k))
    equations = iron.Equations()
    equationsSet.EquationsCreateStart(equations)
    equations.sparsityType = iron.EquationsSparsityTypes.SPARSE
    equations.outputType = iron.EquationsOutputTypes.NONE
    equationsSet.EquationsCreateFinish()
    problem = iron.Problem()
    problem.CreateStart(12, [iron.ProblemClasses.CLASSICAL_FIELD, iron.ProblemTypes.LAPLACE_EQUATION,
                             iron.ProblemSubtypes.STANDARD_LAPLACE])
    problem.CreateFinish()
    problem.ControlLoopCreateStart()
    problem.ControlLoopCreateFinish()
    solver = iron.Solver()
    problem.SolversCreateStart()
    problem.SolverGet([iron.ControlLoopIdentifiers.NODE], 1, solver)
    solver.outputType = iron.SolverOutputTypes.SOLVER
    solver.linearType = iron.LinearSolverTypes.ITERATIVE
    solver.linearIterativeAbsoluteTolerance = 1.0E-12
    solver.linearIterativeRelativeTolerance = 1.0E-12
    problem.SolversCreateFinish()
    solver = iron.Solver()
    solverEquations = iron.SolverEquations()
    problem.SolverEquationsCreateStart()
    problem.SolverGet([iron.ControlLoopIdentifiers.NODE], 1, solver)
    solver.SolverEquationsGet(solverEquations)
    solverEquations.sparsityType = iron.SolverEquationsSparsityTypes.SPARSE
    solverEquations.EquationsSetAdd(equationsSet)
    problem.SolverEquationsCreateFinish()
    boundaryConditions = iron.BoundaryConditions()
    solverEquations.BoundaryConditionsCreateStart(boundaryConditions)
    nodes = iron.Nodes()
    region.NodesGet(nodes)
    last = nodes.numberOfNodes
    assert decomposition.NodeDomainGet(1, 1) == iron.ComputationalNodeNumberGet()
    boundaryConditions.SetNode(dependentField, iron.FieldVariableTypes.U, 1, 1, 1, 1,
                               iron.BoundaryConditionsTypes.FIXED, 0.0)
    boundaryConditions.SetNode(dependentField, iron.FieldVariableTypes.U, 1, 1, last, 1,
                               iron.BoundaryConditionsTypes.FIXED, 1.0)
    solverEquations.BoundaryConditionsCreateFinish()
    problem.Solve()
    u = np.array([dependentField.ParameterSetGetNodeDP(iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES,
                                                       1, 1, k + 1, 1) for k in range(last)])
    K = iron.DistributedMatrix()
    equations.LinearMatrixGet(1, K)
    rp, ci = K.StorageLocationsGet()
    return u, (rp, ci, K.DataGet()), (n, width, height, length), problem


def _oracle_laplace(n, width, height, length, kappa):
    en = oracle.regular_mesh([n, n, n], 1)
    xyz = oracle.regular_coords([n, n, n], 1, [0, 0, 0], [width, height, length])
    N = xyz.shape[1]
    rp, ci = oracle.csr_structure(en, N)
    vals, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], en, xyz, kappa, rp, ci)
    fixed = np.zeros(N, np.uint8)
    fixed[0] = fixed[-1] = 1
    x0 = np.zeros(N)
    x0[-1] = 1.0
    u, _, _ = oracle.cg_dirichlet(rp, ci, vals, None, fixed, x0, rtol=1e-14)
    return u, (rp, ci, vals)


@pytest.mark.parametrize("generalised", [False, True])
def test_laplace_example_sequence_matches_oracle(gfe_cuda, generalised):
    kappa = cond = None
    subtype = iron.EquationsSetSubtypes.STANDARD_LAPLACE
    if generalised:
        kappa = np.exp(np.random.default_rng(4).uniform(np.log(0.1), np.log(10.0), 125))
        cond = np.vstack([kappa, kappa, kappa, np.zeros((3, 125))])
        subtype = iron.EquationsSetSubtypes.GENERALISED_LAPLACE
    u, (rp, ci, vals), dims, _ = _laplace_sequence(subtype, cond)
    uo, (orp, oci, ovals) = _oracle_laplace(*dims, kappa)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(vals - ovals).max() <= 1e-13 * np.abs(ovals).max()
    assert u[0] == 0.0 and u[-1] == 1.0
    assert np.abs(u - uo).max() <= 1e-9 * np.abs(uo).max()


def test_generalised_laplace_with_fibre_field_matches_oracle(gfe_cuda):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    n = 4
    rng = np.random.default_rng(8)
    L = rng.normal(size=(n ** 3, 3, 3))
    T = L @ L.transpose(0, 2, 1) + 0.3 * np.eye(3)
    cond = np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], T[:, 0, 1], T[:, 1, 2], T[:, 0, 2]])
    fibre = rng.uniform(-0.8, 0.8, (3, (n + 1) ** 3))
    u, (rp, ci, vals), (n, width, height, length), _ = _laplace_sequence(
        iron.EquationsSetSubtypes.GENERALISED_LAPLACE, cond, n=n, fibre=fibre)
    en = oracle.regular_mesh([n, n, n], 1)
    xyz = oracle.regular_coords([n, n, n], 1, [0, 0, 0], [width, height, length])
    N = xyz.shape[1]
    orp, oci = oracle.csr_structure(en, N)
    ovals, _ = oracle.laplace_generalised_assemble(3, [1, 1, 1], [2, 2, 2], en, xyz, cond.T.copy(), orp, oci, fibre)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(vals - ovals).max() <= 1e-13 * np.abs(ovals).max()
    # the oracle's system solved directly: u = 0 at the first node, 1 at the last
    K = sp.csr_matrix((ovals, oci - 1, orp - 1), shape=(N, N))
    free = np.ones(N, bool)
    free[[0, N - 1]] = False
    x = np.zeros(N)
    x[-1] = 1.0
    x[free] = sla.spsolve(K[free][:, free].tocsc(), -K[free][:, ~free] @ x[~free])
    assert u[0] == 0.0 and u[-1] == 1.0
    assert np.abs(u - x).max() <= 1e-9 * np.abs(x).max()


def test_context_mesh_cache_shares_structure(gfe_cuda):
    from iron_gb300.context import Context

    ctx = Context()
    a = ctx.regular_mesh(4, 3, 2)
    b = ctx.regular_mesh(4, 3, 2)
    assert ctx.cached_meshes() == 1
    ra, _ = a.csr()
    rb, _ = b.csr()
    assert ra.data_ptr() == rb.data_ptr()
    m = M.RegularMesh((4, 3, 2))
    c = ctx.mesh(m.elem_nodes, m.n_nodes)  # same connectivity given explicitly: a general mesh entry
    assert ctx.cached_meshes() == 2
    rc_, cc = c.csr()
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    assert np.array_equal(rc_.cpu().numpy(), rp) and np.array_equal(cc.cpu().numpy(), ci)
    d = ctx.mesh(m.elem_nodes, m.n_nodes)
    assert ctx.cached_meshes() == 2 and d.csr()[0].data_ptr() == rc_.data_ptr()
    # the context's error word: a degenerate element (its x = 1 face collapsed onto its x = 0 face,
    # so dx/dxi1 = 0 and det GL = 0) raises on it, not on the library word.  An inverted element
    # is integrated like Iron does, with Jacobian sqrt|det GL| > 0 (src/coordinate_routines.F90:818-822).
    coords = torch.from_numpy(m.coords.copy()).cuda()
    en0 = torch.from_numpy(m.elem_nodes[0].astype(np.int64)).cuda()
    coords[:, en0[[1, 3, 5, 7]]] = coords[:, en0[[0, 2, 4, 6]]]
    vals = torch.empty(c.nnz, dtype=torch.float64, device="cuda")
    from iron_gb300 import _lib
    _lib.device_errors()
    with pytest.raises(_lib.GfeError, match="non-positive Jacobian"):
        c.assemble_laplace(coords, None, vals)
    assert _lib.device_errors() == 0
    for h in (a, b, c, d):
        h.close()
    ctx.close()


def _mr_sequence(jacobian_type, n=(2, 2, 2), lam=1.1, increments=3):
    c10, c01 = 2.0, 6.0
    width, length, height = 1.0, 1.0, 1.0
    coordinateSystem = iron.CoordinateSystem()
    coordinateSystem.CreateStart(1)
    coordinateSystem.DimensionSet(3)
    coordinateSystem.CreateFinish()
    region = iron.Region()
    region.CreateStart(1, iron.WorldRegion)
    region.LabelSet("Region")
    region.coordinateSystem = coordinateSystem
    region.CreateFinish()
    basis = iron.Basis()
    basis.CreateStart(1)
    basis.type = iron.BasisTypes.LAGRANGE_HERMITE_TP
    basis.numberOfXi = 3
    basis.interpolationXi = [iron.BasisInterpolationSpecifications.QUADRATIC_LAGRANGE] * 3
    basis.quadratureNumberOfGaussXi = [3] * 3
    basis.CreateFinish()
    pressureBasis = iron.Basis()
    pressureBasis.CreateStart(2)
    pressureBasis.type = iron.BasisTypes.LAGRANGE_HERMITE_TP
    pressureBasis.numberOfXi = 3
    pressureBasis.interpolationXi = [iron.BasisInterpolationSpecifications.LINEAR_LAGRANGE] * 3
    pressureBasis.quadratureNumberOfGaussXi = [3] * 3
    pressureBasis.CreateFinish()
    generatedMesh = iron.GeneratedMesh()
    generatedMesh.CreateStart(1, region)
    generatedMesh.type = iron.GeneratedMeshTypes.REGULAR
    generatedMesh.basis = [basis, pressureBasis]
    generatedMesh.extent = [width, length, height]
    generatedMesh.numberOfElements = list(n)
    mesh = iron.Mesh()
    generatedMesh.CreateFinish(1, mesh)
    decomposition = iron.Decomposition()
    decomposition.CreateStart(1, mesh)
    decomposition.type = iron.DecompositionTypes.CALCULATED
    decomposition.numberOfDomains = 1
    decomposition.CreateFinish()
    geometricField = iron.Field()
    geometricField.CreateStart(1, region)
    geometricField.MeshDecompositionSet(decomposition)
    geometricField.TypeSet(iron.FieldTypes.GEOMETRIC)
    for c in (1, 2, 3):
        geometricField.ComponentMeshComponentSet(iron.FieldVariableTypes.U, c, 1)
    geometricField.CreateFinish()
    generatedMesh.GeometricParametersCalculate(geometricField)
    fibreField = iron.Field()
    fibreField.CreateStart(2, region)
    fibreField.TypeSet(iron.FieldTypes.FIBRE)
    fibreField.MeshDecompositionSet(decomposition)
    fibreField.GeometricFieldSet(geometricField)
    fibreField.CreateFinish()
    equationsSetField = iron.Field()
    equationsSet = iron.EquationsSet()
    spec = [iron.EquationsSetClasses.ELASTICITY, iron.EquationsSetTypes.FINITE_ELASTICITY,
            iron.EquationsSetSubtypes.MOONEY_RIVLIN]
    equationsSet.CreateStart(1, region, fibreField, spec, 6, equationsSetField)
    equationsSet.CreateFinish()
    dependentField = iron.Field()
    equationsSet.DependentCreateStart(4, dependentField)
    dependentField.ComponentMeshComponentSet(iron.FieldVariableTypes.U, 4, 2)
    equationsSet.DependentCreateFinish()
    for c in (1, 2, 3):
        iron.Field.ParametersToFieldParametersComponentCopy(
            geometricField, iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES, c,
            dependentField, iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES, c)
    iron.Field.ComponentValuesInitialiseDP(dependentField, iron.FieldVariableTypes.U,
                                           iron.FieldParameterSetTypes.VALUES, 4, 0.0)
    materialField = iron.Field()
    equationsSet.MaterialsCreateStart(3, materialField)
    equationsSet.MaterialsCreateFinish()
    materialField.ComponentValuesInitialiseDP(iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES, 1, c10)
    materialField.ComponentValuesInitialiseDP(iron.FieldVariableTypes.U, iron.FieldParameterSetTypes.VALUES, 2, c01)
    equations = iron.Equations()
    equationsSet.EquationsCreateStart(equations)
    equations.sparsityType = iron.EquationsSparsityTypes.SPARSE
    equations.outputType = iron.EquationsOutputTypes.NONE
    if jacobian_type is not None:
        equations.JacobianCalculationTypeSet(1, iron.FieldVariableTypes.U, jacobian_type)
    equationsSet.EquationsCreateFinish()
    problem = iron.Problem()
    problem.CreateStart(1, [iron.ProblemClasses.ELASTICITY, iron.ProblemTypes.FINITE_ELASTICITY,
                            iron.ProblemSubtypes.NONE])
    problem.CreateFinish()
    problem.ControlLoopCreateStart()
    controlLoop = iron.ControlLoop()
    problem.ControlLoopGet([iron.ControlLoopIdentifiers.NODE], controlLoop)
    controlLoop.MaximumIterationsSet(increments)
    problem.ControlLoopCreateFinish()
    nonLinearSolver = iron.Solver()
    linearSolver = iron.Solver()
    problem.SolversCreateStart()
    problem.SolverGet([iron.ControlLoopIdentifiers.NODE], 1, nonLinearSolver)
    nonLinearSolver.outputType = iron.SolverOutputTypes.PROGRESS
    nonLinearSolver.NewtonJacobianCalculationTypeSet(iron.JacobianCalculationTypes.EQUATIONS)
    nonLinearSolver.NewtonAbsoluteToleranceSet(1e-12)
    nonLinearSolver.NewtonRelativeToleranceSet(1e-14)
    nonLinearSolver.NewtonLinearSolverGet(linearSolver)
    linearSolver.linearType = iron.LinearSolverTypes.DIRECT
    problem.SolversCreateFinish()
    solver = iron.Solver()
    solverEquations = iron.SolverEquations()
    problem.SolverEquationsCreateStart()
    problem.SolverGet([iron.ControlLoopIdentifiers.NODE], 1, solver)
    solver.SolverEquationsGet(solverEquations)
    solverEquations.sparsityType = iron.SolverEquationsSparsityTypes.SPARSE
    solverEquations.EquationsSetAdd(equationsSet)
    problem.SolverEquationsCreateFinish()
    # rollers on x = 0, y = 0, z = 0 and the face x = X pulled to lam X
    boundaryConditions = iron.BoundaryConditions()
    solverEquations.BoundaryConditionsCreateStart(boundaryConditions)
    x = geometricField.values.reshape(3, -1)
    for k in range(x.shape[1]):
        for comp in (1, 2, 3):
            if abs(x[comp - 1, k]) < 1e-12:
                boundaryConditions.AddNode(dependentField, iron.FieldVariableTypes.U, 1, 1, k + 1, comp,
                                           iron.BoundaryConditionsTypes.FIXED, 0.0)
        if abs(x[0, k] - width) < 1e-12:
            boundaryConditions.SetNode(dependentField, iron.FieldVariableTypes.U, 1, 1, k + 1, 1,
                                       iron.BoundaryConditionsTypes.FIXED, lam * width)
    solverEquations.BoundaryConditionsCreateFinish()
    problem.Solve()
    return dependentField, x, (c10, c01, lam)


@pytest.mark.parametrize("jacobian_type", [None, iron.EquationsJacobianCalculated.CONSISTENT])
def test_mooney_rivlin_example_sequence_reaches_uniaxial_stretch(gfe_cuda, jacobian_type):
    dep, x, (c10, c01, lam) = _mr_sequence(jacobian_type)
    nq = x.shape[1]
    z = dep.values[: 3 * nq].reshape(3, nq)
    exact = x * np.array([lam, lam ** -0.5, lam ** -0.5])[:, None]
    assert np.abs(z - exact).max() <= 1e-9 * np.abs(exact).max()
    F = np.diag([lam, lam ** -0.5, lam ** -0.5])
    Cb = F.T @ F
    sb = F @ (2.0 * (c10 + np.trace(Cb) * c01) * np.eye(3) - 2.0 * c01 * Cb) @ F.T
    p = np.trace(sb) / 3.0 - sb[1, 1]
    assert np.abs(dep.values[3 * nq:] - p).max() <= 1e-8 * abs(p)
