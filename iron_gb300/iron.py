"""Iron-shaped Python surface for the hot path's subset of OpenCMISS-Iron's `opencmiss.iron` API.

A script written against Iron's Python bindings for the configurations this package covers runs
against `from iron_gb300 import iron` with the same object names, Create/Finish sequence,
properties and enumerations (bindings/python/tests/Laplace.py:99-187 and Cantilever.py are the
models), and `problem.Solve()` runs the element loop, structure and solve on the GPU:

- classical field, Laplace equation, standard or generalised subtype on Iron's regular generated
  mesh of trilinear-Lagrange hexahedra with 2x2x2 Gauss points.  The generalised materials field
  has Iron's six components K11 K22 K33 K12 K23 K13 (constants or element values), and a fibre
  field (FieldTypes.FIBRE, up to three node-based angles) passed to EquationsSet.CreateStart
  as Iron's geometric-fibre field sets the material frame.  An isotropic tensor runs the standard
  element loop with a per-element conductivity (GPU context / mesh-handle path, Jacobi-CG); any
  other tensor runs the generalised element loop, whose matrix is not symmetric, and restarted
  GMRES (Iron's default Krylov method);
- elasticity, finite elasticity, Mooney-Rivlin subtype on a regular generated mesh of
  triquadratic-Lagrange displacement with a trilinear pressure basis (two mesh components,
  node-based pressure), 3x3x3 Gauss points, load-stepped Newton with the Jacobian type chosen by
  `equations.JacobianCalculationTypeSet` (Iron's default for finite elasticity is finite
  differences) and the step by `equations.JacobianFiniteDifferenceStepSizeSet`.

Errors raise `CMFEError` with the library's message, as Iron's bindings do on a non-zero status
(bindings/python/opencmiss/iron/_utils.in.py:27-78).  Calls the subset does not cover raise
`CMFEError` naming what is unsupported instead of computing something else.  Enumeration values are
Iron's (src/opencmiss_iron.F90 constants) so that values stored by a user script mean the same.
"""
from __future__ import annotations

import functools

import numpy as np
import torch

from . import _lib
from ._lib import GfeError


class CMFEError(Exception):
    """Raised for a non-zero status of the library, like Iron's bindings."""


class CMFEType(object):
    """Base class of the handle types."""


class Enum(object):
    pass


def _wrap(fn):
    @functools.wraps(fn)
    def inner(*a, **k):
        try:
            return fn(*a, **k)
        except GfeError as e:
            raise CMFEError(str(e)) from e
    return inner


def _fail(msg: str):
    raise CMFEError(msg)


# -- enumerations (Iron's values) -------------------------------------------------------------
class BasisTypes(Enum):
    LAGRANGE_HERMITE_TP = 1
    SIMPLEX = 2


class BasisInterpolationSpecifications(Enum):
    LINEAR_LAGRANGE = 1
    QUADRATIC_LAGRANGE = 2
    CUBIC_LAGRANGE = 3
    CUBIC_HERMITE = 4
    LINEAR_SIMPLEX = 7
    QUADRATIC_SIMPLEX = 8
    CUBIC_SIMPLEX = 9


class GeneratedMeshTypes(Enum):
    REGULAR = 1
    POLAR = 2
    FRACTAL_TREE = 3
    CYLINDER = 4
    ELLIPSOID = 5


class DecompositionTypes(Enum):
    ALL = 1
    CALCULATED = 2
    USER_DEFINED = 3


class FieldTypes(Enum):
    GEOMETRIC = 1
    FIBRE = 2
    GENERAL = 3
    MATERIAL = 4


class FieldVariableTypes(Enum):
    U = 1
    DELUDELN = 2
    DELUDELT = 3
    DEL2UDELT2 = 4
    V = 5


class FieldParameterSetTypes(Enum):
    VALUES = 1


class FieldDOFOrderTypes(Enum):
    SEPARATED = 1
    CONTIGUOUS = 2


class FieldInterpolationTypes(Enum):
    CONSTANT = 1
    ELEMENT_BASED = 2
    NODE_BASED = 3


class FieldScalingTypes(Enum):
    NONE = 0
    UNIT = 1
    ARC_LENGTH = 2
    ARITHMETIC_MEAN = 3
    GEOMETRIC_MEAN = 4
    HARMONIC_MEAN = 5


class EquationsSetClasses(Enum):
    ELASTICITY = 1
    CLASSICAL_FIELD = 4


class EquationsSetTypes(Enum):
    """Values are scoped by class in Iron (src/equations_set_constants.F90:69, 84): the
    specification list [class, type, subtype] identifies an equations set."""
    LAPLACE_EQUATION = 1
    FINITE_ELASTICITY = 2


class EquationsSetSubtypes(Enum):
    STANDARD_LAPLACE = 1
    GENERALISED_LAPLACE = 2
    MOONEY_RIVLIN = 1


class ProblemClasses(Enum):
    ELASTICITY = 1
    CLASSICAL_FIELD = 4


class ProblemTypes(Enum):
    LAPLACE_EQUATION = 1
    FINITE_ELASTICITY = 2


class ProblemSubtypes(Enum):
    NONE = 0
    STANDARD_LAPLACE = 1


class EquationsSparsityTypes(Enum):
    SPARSE = 1
    FULL = 2


class EquationsOutputTypes(Enum):
    NONE = 0
    TIMING = 1
    MATRIX = 2
    ELEMENT_MATRIX = 3


class EquationsJacobianCalculated(Enum):
    """cmfe_Equations_JacobianCalculationTypeSet values (src/opencmiss_iron.F90:2301-2302); CONSISTENT
    (the exact derivative of the residual) is this package's addition."""
    FINITE_DIFFERENCE = 1
    ANALYTIC = 2
    CONSISTENT = 100


class JacobianCalculationTypes(Enum):
    """cmfe_Solver_NewtonJacobianCalculationTypeSet values (src/opencmiss_iron.F90:6584-6586)."""
    NOT_CALCULATED = 1
    EQUATIONS = 2
    FD = 3


class ControlLoopIdentifiers(Enum):
    NODE = 0


class SolverOutputTypes(Enum):
    NONE = 0
    PROGRESS = 1
    TIMING = 2
    SOLVER = 3
    MATRIX = 4


class LinearSolverTypes(Enum):
    DIRECT = 1
    ITERATIVE = 2


class SolverEquationsSparsityTypes(Enum):
    SPARSE = 1
    FULL = 2


class BoundaryConditionsTypes(Enum):
    FREE = 0
    FIXED = 1


# -- library-level routines ----------------------------------------------------------------
def ComputationalNumberOfNodesGet() -> int:
    """One process per GPU: the distributed element loop is not in this package's scope."""
    return 1


def ComputationalNodeNumberGet() -> int:
    return 0


def DiagnosticsSetOn(*args) -> None:
    """Iron's diagnostics output is not reproduced; accepted and ignored."""


def Finalise() -> None:
    torch.cuda.synchronize() if torch.cuda.is_available() else None


# -- handle types ------------------------------------------------------------------------------
class CoordinateSystem(CMFEType):
    def __init__(self):
        self.dimension = 3
        self.finished = False

    def CreateStart(self, user_number: int):
        self.user_number = user_number

    def DimensionSet(self, d: int):
        self.dimension = d

    def CreateFinish(self):
        if self.dimension != 3:
            _fail("only three-dimensional coordinate systems are covered")
        self.finished = True


class Region(CMFEType):
    def __init__(self):
        self.label = ""
        self.coordinateSystem = None
        self.generated_mesh = None

    def CreateStart(self, user_number: int, parent):
        self.user_number = user_number
        self.parent = parent

    def LabelSet(self, label: str):
        self.label = label

    def CoordinateSystemSet(self, cs):
        self.coordinateSystem = cs

    def CreateFinish(self):
        if self.coordinateSystem is None:
            _fail("region has no coordinate system")

    def NodesGet(self, nodes: "Nodes"):
        gm = self.generated_mesh
        if gm is None:
            _fail("region has no mesh")
        nodes.numberOfNodes = gm.number_of_nodes()


WorldRegion = Region()


class Nodes(CMFEType):
    def __init__(self):
        self.numberOfNodes = 0


class Basis(CMFEType):
    def __init__(self):
        self.type = BasisTypes.LAGRANGE_HERMITE_TP
        self.numberOfXi = 3
        self.interpolationXi = [BasisInterpolationSpecifications.LINEAR_LAGRANGE] * 3
        self.quadratureNumberOfGaussXi = None

    def CreateStart(self, user_number: int):
        self.user_number = user_number

    def CreateFinish(self):
        if self.type != BasisTypes.LAGRANGE_HERMITE_TP or self.numberOfXi != 3:
            _fail("covered bases: three-dimensional tensor-product Lagrange")
        if len(set(self.interpolationXi)) != 1 or self.interpolationXi[0] not in (1, 2):
            _fail("covered bases: trilinear or triquadratic Lagrange")
        order = self.interpolationXi[0]
        if self.quadratureNumberOfGaussXi is None:
            self.quadratureNumberOfGaussXi = [order + 1] * 3
        self.order = order


class Mesh(CMFEType):
    pass


class GeneratedMesh(CMFEType):
    def __init__(self):
        self.type = GeneratedMeshTypes.REGULAR
        self.basis = []
        self.extent = [1.0, 1.0, 1.0]
        self.numberOfElements = [1, 1, 1]
        self.origin = [0.0, 0.0, 0.0]

    def CreateStart(self, user_number: int, region: Region):
        self.user_number = user_number
        self.region = region

    def CreateFinish(self, mesh_user_number: int, mesh: Mesh):
        if self.type != GeneratedMeshTypes.REGULAR:
            _fail("covered generated meshes: REGULAR")
        if not self.basis or len(self.numberOfElements) != 3:
            _fail("a regular generated mesh needs a basis and three element counts")
        self.mesh = mesh
        mesh.generated = self
        self.region.generated_mesh = self

    @property
    def order(self) -> int:
        return self.basis[0].order

    def number_of_nodes(self) -> int:
        return int(np.prod([self.order * n + 1 for n in self.numberOfElements]))

    def GeometricParametersCalculate(self, field: "Field"):
        from .mesh import regular_coords

        field.values = regular_coords(tuple(self.numberOfElements), self.order, tuple(self.origin),
                                      tuple(self.extent)).reshape(-1).copy()
        field.generated_mesh = self


class Decomposition(CMFEType):
    def __init__(self):
        self.type = DecompositionTypes.CALCULATED
        self.numberOfDomains = 1

    def CreateStart(self, user_number: int, mesh: Mesh):
        self.mesh = mesh

    def CreateFinish(self):
        if self.numberOfDomains != 1:
            _fail("one domain per GPU: decompositions over several domains are not covered")

    def NodeDomainGet(self, node: int, mesh_component: int) -> int:
        return 0


class Field(CMFEType):
    def __init__(self):
        self.values = None
        self.element_values = {}
        self.fieldScalingType = FieldScalingTypes.UNIT
        self.role = None
        self.labels = {}
        self.meshDecomposition = None

    def CreateStart(self, user_number: int, region: Region):
        self.user_number = user_number
        self.region = region

    def MeshDecompositionSet(self, d):
        self.meshDecomposition = d

    def TypeSet(self, t):
        self.type = t

    def VariableLabelSet(self, var, label):
        self.labels[var] = label

    def GeometricFieldSet(self, f):
        self.geometric = f

    def ComponentMeshComponentSet(self, var, comp, mesh_comp):
        pass

    def ComponentInterpolationSet(self, var, comp, interp):
        self.interpolation = getattr(self, "interpolation", {})
        self.interpolation[(var, int(comp))] = interp

    def DOFOrderTypeSet(self, var, order):
        if order != FieldDOFOrderTypes.SEPARATED:
            _fail("covered DOF order: separated (Iron's default for these fields)")

    def NumberOfComponentsSet(self, var, n):
        self.n_components = int(n)

    def CreateFinish(self):
        if getattr(self, "type", None) == FieldTypes.FIBRE:
            # node-based fibre angles on the geometric mesh; Iron's default: one per dimension
            gm = getattr(self.region, "generated_mesh", None)
            if gm is None:
                _fail("a fibre field needs the region's generated mesh")
            nc = getattr(self, "n_components", 3)
            if not 1 <= nc <= 3:
                _fail("a fibre field has 1 to 3 angle components")
            n = gm.number_of_nodes()
            self.role = "fibre"
            self.values = np.zeros(nc * n)
            self.layout = lambda comp: ((comp - 1) * n, comp * n)
            self.node_dof = lambda node, comp: (comp - 1) * n + node - 1

    # parameter access on the dependent / materials vectors, Iron's 1-based numbers
    def _layout(self):
        lay = getattr(self, "layout", None)
        if lay is None:
            _fail("field has no parameters yet")
        return lay

    @_wrap
    def ComponentValuesInitialiseDP(self, var, set_type, comp, value):
        if self.role == "materials":
            self.constants[comp] = float(value)
            return
        lo, hi = self._layout()(comp)
        self.values[lo:hi] = value

    @_wrap
    def ParameterSetGetNodeDP(self, var, set_type, version, deriv, node, comp) -> float:
        return float(self.values[self._node_dof(node, comp)])

    @_wrap
    def ParameterSetUpdateNodeDP(self, var, set_type, version, deriv, node, comp, value):
        self.values[self._node_dof(node, comp)] = value

    @_wrap
    def ParameterSetUpdateElementDP(self, var, set_type, element, comp, value):
        self.element_values.setdefault(comp, {})[int(element)] = float(value)

    def _node_dof(self, node, comp) -> int:
        fn = getattr(self, "node_dof", None)
        if fn is None:
            _fail("field has no node-based parameters")
        return fn(int(node), int(comp))

    @staticmethod
    def ParametersToFieldParametersComponentCopy(src, src_var, src_set, src_comp, dst, dst_var, dst_set, dst_comp):
        n = src.values.size // 3
        lo, hi = dst._layout()(dst_comp)
        dst.values[lo:hi] = src.values[(src_comp - 1) * n:src_comp * n]


class EquationsSet(CMFEType):
    def CreateStart(self, user_number, region, geometric_field, specification, field_user_number, field):
        self.user_number = user_number
        self.region = region
        self.geometric = getattr(geometric_field, "geometric", geometric_field)
        # Iron's geometric-fibre argument: a fibre field carries the material frame's angles
        self.fibre = geometric_field if getattr(geometric_field, "type", None) == FieldTypes.FIBRE else None
        spec = list(specification)
        if len(spec) != 3:
            _fail("an equations set specification is [class, type, subtype]")
        if spec[:2] == [EquationsSetClasses.CLASSICAL_FIELD, EquationsSetTypes.LAPLACE_EQUATION] and \
                spec[2] in (EquationsSetSubtypes.STANDARD_LAPLACE, EquationsSetSubtypes.GENERALISED_LAPLACE):
            self.kind = "laplace"
        elif spec[:2] == [EquationsSetClasses.ELASTICITY, EquationsSetTypes.FINITE_ELASTICITY] and \
                spec[2] == EquationsSetSubtypes.MOONEY_RIVLIN:
            self.kind = "mooney_rivlin"
        else:
            _fail(f"equations set {spec} is outside the covered subset (standard / generalised Laplace, "
                  "Mooney-Rivlin finite elasticity)")
        self.subtype = spec[2]
        self.materials = None
        self.equations = None

    def CreateFinish(self):
        gm = self.geometric.generated_mesh
        if self.kind == "laplace" and (gm.order != 1 or list(gm.basis[0].quadratureNumberOfGaussXi) != [2, 2, 2]):
            _fail("the Laplace element loop covers trilinear hexahedra with 2x2x2 Gauss points")
        if self.kind == "mooney_rivlin" and any(float(v) != 0.0 for v in gm.origin):
            _fail("Mooney-Rivlin meshes are generated at the origin")
        if self.kind == "mooney_rivlin" and (gm.order != 2 or len(gm.basis) != 2 or gm.basis[1].order != 1):
            _fail("Mooney-Rivlin covers triquadratic displacement with a trilinear pressure basis (mesh components 1, 2)")

    def DependentCreateStart(self, user_number, field: Field):
        self.dependent = field
        field.role = "dependent"
        gm = self.geometric.generated_mesh
        if self.kind == "laplace":
            n = gm.number_of_nodes()
            field.values = np.zeros(n)
            field.layout = lambda comp: (0, n)
            field.node_dof = lambda node, comp: node - 1
        else:
            from .elasticity import _regular_q2_mesh

            m, elin, lin2g, _, _ = _regular_q2_mesh(tuple(gm.numberOfElements), tuple(float(v) for v in gm.extent))
            nq, nl = m.n_nodes, len(lin2g)
            g2l = {int(g): i for i, g in enumerate(lin2g)}
            field.values = np.zeros(3 * nq + nl)
            field.layout = lambda comp: ((comp - 1) * nq, comp * nq) if comp <= 3 else (3 * nq, 3 * nq + nl)

            def node_dof(node, comp):
                if comp <= 3:
                    return (comp - 1) * nq + node - 1
                if node - 1 not in g2l:
                    _fail(f"node {node} carries no pressure (not a corner of the pressure mesh component)")
                return 3 * nq + g2l[node - 1]
            field.node_dof = node_dof

    def DependentCreateFinish(self):
        interp = getattr(self.dependent, "interpolation", {})
        for (var, comp), how in interp.items():
            if how != FieldInterpolationTypes.NODE_BASED:
                _fail("covered dependent field components: node based (element-based pressure is not covered)")

    def MaterialsCreateStart(self, user_number, field: Field):
        self.materials = field
        field.role = "materials"
        field.constants = {}

    def MaterialsCreateFinish(self):
        pass

    def SourceCreateStart(self, user_number, field: Field):
        _fail("source fields (body forces) are not covered")

    def EquationsCreateStart(self, equations: "Equations"):
        self.equations = equations
        equations.equations_set = self
        # Iron's default Jacobian for finite elasticity is finite differences
        equations.jacobian_type = EquationsJacobianCalculated.FINITE_DIFFERENCE
        equations.fd_step = 1e-6

    def EquationsCreateFinish(self):
        if self.equations.sparsityType != EquationsSparsityTypes.SPARSE:
            _fail("covered equations storage: sparse (compressed row)")


class DistributedMatrix(CMFEType):
    def __init__(self):
        self.csr = None

    def StorageLocationsGet(self):
        """(rowIndices, columnIndices) of the compressed-row storage, 1-based as Iron's
        cmfe_DistributedMatrix_StorageLocationsGet (src/opencmiss_iron.F90:45823)."""
        return self.csr[0].copy(), self.csr[1].copy()

    def DataGet(self):
        """The FP64 values (cmfe_DistributedMatrix_DataGet, src/opencmiss_iron.F90:45903)."""
        return self.csr[2].copy()


class Equations(CMFEType):
    def __init__(self):
        self.sparsityType = EquationsSparsityTypes.SPARSE
        self.outputType = EquationsOutputTypes.NONE
        self.jacobian_type = EquationsJacobianCalculated.FINITE_DIFFERENCE
        self.fd_step = 1e-6
        self.matrix = None

    def JacobianCalculationTypeSet(self, residual_index, variable_type, calculation_type):
        if calculation_type not in (1, 2, 100):
            _fail(f"unknown Jacobian calculation type {calculation_type}")
        self.jacobian_type = calculation_type

    def JacobianFiniteDifferenceStepSizeSet(self, residual_index, variable_type, step):
        if not step > 0.0:
            _fail("the finite-difference step must be positive")
        self.fd_step = float(step)

    def LinearMatrixGet(self, index: int, matrix: DistributedMatrix):
        if self.matrix is None:
            _fail("the equations have not been assembled (call problem.Solve())")
        matrix.csr = self.matrix

    JacobianMatrixGet = LinearMatrixGet


class ControlLoop(CMFEType):
    def __init__(self):
        self.maximum_iterations = 1

    def MaximumIterationsSet(self, n):
        self.maximum_iterations = int(n)


class Solver(CMFEType):
    def __init__(self):
        self.outputType = SolverOutputTypes.NONE
        self.linearType = LinearSolverTypes.ITERATIVE
        self.linearIterativeAbsoluteTolerance = 1e-10
        self.linearIterativeRelativeTolerance = 1e-5
        self.linearIterativeMaximumIterations = 100000
        self.newtonAbsoluteTolerance = 1e-10
        self.newtonRelativeTolerance = 1e-5
        self.newtonMaximumIterations = 50
        self.newton_jacobian = JacobianCalculationTypes.EQUATIONS
        self.problem = None

    def _bind(self, problem, shared):
        self.__dict__ = shared.__dict__  # every SolverGet of the same solver returns one state
        self.problem = problem

    def SolverEquationsGet(self, se: "SolverEquations"):
        se.__dict__ = self.problem.solver_equations.__dict__

    def NewtonJacobianCalculationTypeSet(self, t):
        self.newton_jacobian = t

    def NewtonLinearSolverGet(self, linear: "Solver"):
        linear.__dict__ = self.__dict__

    def NewtonAbsoluteToleranceSet(self, v):
        self.newtonAbsoluteTolerance = float(v)

    def NewtonRelativeToleranceSet(self, v):
        self.newtonRelativeTolerance = float(v)

    def NewtonMaximumIterationsSet(self, v):
        self.newtonMaximumIterations = int(v)


class SolverEquations(CMFEType):
    def __init__(self):
        self.sparsityType = SolverEquationsSparsityTypes.SPARSE
        self.equations_sets = []
        self.boundary_conditions = None

    def EquationsSetAdd(self, es: EquationsSet) -> int:
        if self.equations_sets:
            _fail("one equations set per solver equations is covered")
        self.equations_sets.append(es)
        return 1

    def BoundaryConditionsCreateStart(self, bc: "BoundaryConditions"):
        self.boundary_conditions = bc
        bc.entries = []

    def BoundaryConditionsCreateFinish(self):
        pass


class BoundaryConditions(CMFEType):
    """Dirichlet conditions on the dependent field (cmfe_BoundaryConditions_SetNode / AddNode):
    SetNode fixes a DOF at `value`, AddNode at its current value plus `value`.  The field keeps
    its value from before the condition, from which load steps increment to the fixed value."""

    def __init__(self):
        self.entries = []

    def _node(self, field, var, node, comp, condition, value, add):
        if condition != BoundaryConditionsTypes.FIXED or var != FieldVariableTypes.U:
            _fail("covered boundary conditions: FIXED values of the U variable")
        k = field._node_dof(int(node), int(comp))
        before = float(field.values[k])
        target = before + float(value) if add else float(value)
        self.entries.append((field, k, before, target))

    def SetNode(self, field, var, version, deriv, node, comp, condition, value):
        self._node(field, var, node, comp, condition, value, False)

    def AddNode(self, field, var, version, deriv, node, comp, condition, value):
        self._node(field, var, node, comp, condition, value, True)


class Problem(CMFEType):
    def __init__(self):
        self.solver_equations = SolverEquations()
        self.solver = Solver()
        self.control_loop = ControlLoop()

    def CreateStart(self, user_number, specification):
        self.specification = list(specification)

    def CreateFinish(self):
        pass

    def ControlLoopCreateStart(self):
        pass

    def ControlLoopGet(self, identifiers, loop: ControlLoop):
        loop.__dict__ = self.control_loop.__dict__

    def ControlLoopCreateFinish(self):
        pass

    def SolversCreateStart(self):
        pass

    def SolverGet(self, identifiers, index, solver: Solver):
        solver._bind(self, self.solver)

    def SolversCreateFinish(self):
        pass

    def SolverEquationsCreateStart(self):
        pass

    def SolverEquationsCreateFinish(self):
        pass

    @_wrap
    def Solve(self):
        se = self.solver_equations
        if not se.equations_sets:
            _fail("no equations set added to the solver equations")
        es = se.equations_sets[0]
        if es.kind == "laplace":
            self._solve_laplace(es, se.boundary_conditions)
        else:
            self._solve_mooney_rivlin(es, se.boundary_conditions)

    def _dirichlet(self, es, bc):
        """(fixed mask, values before the conditions, fixed values) of the dependent vector."""
        dep = es.dependent
        fixed = np.zeros(dep.values.size, np.uint8)
        before = dep.values.copy()
        target = dep.values.copy()
        for field, k, b, t in (bc.entries if bc else []):
            if field is not dep:
                _fail("boundary conditions must be set on the dependent field")
            fixed[k] = 1
            before[k] = b
            target[k] = t
        return fixed, before, target

    def _solve_laplace(self, es, bc):
        from .context import Context

        gm = es.geometric.generated_mesh
        dev = _lib.require_cuda()
        ctx = getattr(self, "_ctx", None) or Context(device=dev)
        self._ctx = ctx
        nx, ny, nz = (int(v) for v in gm.numberOfElements)
        mesh = ctx.regular_mesh(nx, ny, nz)
        coords = torch.from_numpy(es.geometric.values.reshape(3, -1).copy()).to(dev)
        kappa = None
        if es.subtype == EquationsSetSubtypes.GENERALISED_LAPLACE:
            cond = self._conductivity(es, nx * ny * nz)
            if np.all(cond[0] == cond[1]) and np.all(cond[0] == cond[2]) and not np.any(cond[3:]):
                # kappa * I in any frame is kappa * I in xi space: the standard element loop
                kappa = torch.from_numpy(cond[0].copy()).to(dev)
            else:
                return self._solve_laplace_generalised(es, bc, cond)
        values = torch.empty(mesh.nnz, dtype=torch.float64, device=dev)
        mesh.assemble_laplace(coords, kappa, values, "fp64")
        fixed, _, target = self._dirichlet(es, bc)
        dep = es.dependent
        x = torch.from_numpy(np.where(fixed == 1, target, 0.0)).to(dev)
        s = self.solver
        # a DIRECT linear solver is served by the Krylov solver run to a residual near round-off
        rtol = 1e-13 if s.linearType == LinearSolverTypes.DIRECT else float(s.linearIterativeRelativeTolerance)
        mesh.solve(values, torch.from_numpy(fixed).to(dev), x, rtol=rtol,
                   max_iters=int(s.linearIterativeMaximumIterations))
        dep.values[:] = x.cpu().numpy()
        rp, ci = mesh.csr()
        es.equations.matrix = (rp.cpu().numpy(), ci.cpu().numpy(), values.cpu().numpy())

    @staticmethod
    def _conductivity(es, E: int) -> np.ndarray:
        """[6][E] materials components K11 K22 K33 K12 K23 K13: the component constants
        (ComponentValuesInitialiseDP; 0 when unset, as Iron's new field) with element values over them."""
        cond = np.zeros((6, E))
        mat = es.materials
        if mat is None:
            _fail("the generalised Laplace equation needs its materials field")
        if any(c > 6 for c in list(mat.constants) + list(mat.element_values)):
            _fail("the generalised Laplace materials field has 6 components in 3D")
        for c, v in mat.constants.items():
            cond[c - 1] = v
        for c, ev in mat.element_values.items():
            for e, v in ev.items():
                if not 1 <= e <= E:
                    _fail(f"element {e} outside 1..{E}")
                cond[c - 1, e - 1] = v
        return cond

    def _solve_laplace_generalised(self, es, bc, cond):
        from .laplace import LaplaceAssembly
        from .mesh import RegularMesh
        from .newton import gmres_solve

        gm = es.geometric.generated_mesh
        dev = _lib.require_cuda()
        m = RegularMesh(tuple(int(v) for v in gm.numberOfElements))
        A = LaplaceAssembly.from_regular_mesh(m, device=dev)
        A.coords = torch.from_numpy(es.geometric.values.reshape(3, -1).copy()).to(dev)
        fib = None
        if es.fibre is not None:
            fib = es.fibre.values.reshape(-1, m.n_nodes)
        A.assemble_generalised(cond, fib)
        fixed, _, target = self._dirichlet(es, bc)
        x = torch.from_numpy(np.where(fixed == 1, target, 0.0)).to(dev)
        s = self.solver
        rtol = 1e-13 if s.linearType == LinearSolverTypes.DIRECT else float(s.linearIterativeRelativeTolerance)
        f = torch.zeros(A.n_nodes, dtype=torch.float64, device=dev)
        info = gmres_solve(A.row_ptr, A.col_idx, A.values, f, torch.from_numpy(fixed).to(dev), x, rtol=rtol,
                           max_iters=int(s.linearIterativeMaximumIterations))
        if not info.relative_residual <= rtol:
            _fail(f"GMRES stopped at relative residual {info.relative_residual:.3e} after {info.iterations} "
                  "iterations")
        es.dependent.values[:] = x.cpu().numpy()
        es.equations.matrix = (A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy(), A.values.cpu().numpy())

    def _solve_mooney_rivlin(self, es, bc):
        from .elasticity import MooneyRivlinAssembly
        from .newton import NewtonSolver

        gm = es.geometric.generated_mesh
        dev = _lib.require_cuda()
        A = MooneyRivlinAssembly.from_regular_mesh(tuple(int(v) for v in gm.numberOfElements),
                                                   extent=tuple(float(v) for v in gm.extent), device=dev)
        mats = es.materials.constants if es.materials else {}
        c = [mats.get(1, 0.0), mats.get(2, 0.0)]
        eq = es.equations
        s = self.solver
        if s.newton_jacobian == JacobianCalculationTypes.FD:
            jac = "fd"
        elif s.newton_jacobian == JacobianCalculationTypes.EQUATIONS:
            jac = {EquationsJacobianCalculated.FINITE_DIFFERENCE: "fd", EquationsJacobianCalculated.ANALYTIC: "analytic",
                   EquationsJacobianCalculated.CONSISTENT: "consistent"}[eq.jacobian_type]
        else:
            _fail("the Newton solver needs a Jacobian")
        fixed_h, before, target = self._dirichlet(es, bc)
        fixed = torch.from_numpy(fixed_h).to(dev)
        full_vals = torch.from_numpy(target).to(dev)
        # the load steps start from the field before the conditions and move the fixed DOFs to their
        # values in increments (EQUATIONS_SET_BOUNDARY_CONDITIONS_INCREMENT)
        start_t = torch.from_numpy(before.copy()).to(dev)
        solver = NewtonSolver(A, c, jacobian=jac, fd_step=eq.fd_step,
                              absolute_tolerance=s.newtonAbsoluteTolerance,
                              relative_tolerance=s.newtonRelativeTolerance,
                              maximum_iterations=s.newtonMaximumIterations,
                              linear_relative_tolerance=1e-12 if s.linearType == LinearSolverTypes.DIRECT else
                              float(s.linearIterativeRelativeTolerance))
        solver.solve(start_t, fixed, full_vals, load_increments=self.control_loop.maximum_iterations)
        es.dependent.values[:] = start_t.cpu().numpy()
        rp, ci, vals = A.to_iron_csr()
        eq.matrix = (rp, ci, vals)
