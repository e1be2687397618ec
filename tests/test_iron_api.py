"""The Iron-shaped Python surface without a GPU: Iron's enumeration values, the CMFEError mapping
of a library status, and refusals of calls outside the covered subset (before any device work)."""
import pytest

from iron_gb300 import iron
from iron_gb300._lib import GfeError


def test_enumerations_carry_irons_values():
    # src/equations_set_constants.F90, src/problem_constants.F90, src/solver_routines.F90,
    # src/equations_matrices_routines.F90, src/basis_routines.F90
    assert iron.EquationsSetClasses.CLASSICAL_FIELD == 4 and iron.EquationsSetClasses.ELASTICITY == 1
    assert iron.EquationsSetTypes.LAPLACE_EQUATION == 1 and iron.EquationsSetTypes.FINITE_ELASTICITY == 2
    assert iron.EquationsSetSubtypes.GENERALISED_LAPLACE == 2 and iron.EquationsSetSubtypes.MOONEY_RIVLIN == 1
    assert iron.EquationsJacobianCalculated.FINITE_DIFFERENCE == 1 and iron.EquationsJacobianCalculated.ANALYTIC == 2
    assert (iron.JacobianCalculationTypes.NOT_CALCULATED, iron.JacobianCalculationTypes.EQUATIONS,
            iron.JacobianCalculationTypes.FD) == (1, 2, 3)
    assert iron.LinearSolverTypes.DIRECT == 1 and iron.LinearSolverTypes.ITERATIVE == 2
    assert iron.BasisInterpolationSpecifications.CUBIC_HERMITE == 4
    assert iron.BasisInterpolationSpecifications.LINEAR_SIMPLEX == 7


def test_library_status_becomes_cmfe_error():
    @iron._wrap
    def failing():
        raise GfeError(-1, "gfe_x: invalid arguments")

    with pytest.raises(iron.CMFEError, match="invalid arguments"):
        failing()


def test_uncovered_calls_raise_cmfe_error():
    b = iron.Basis()
    b.CreateStart(1)
    b.type = iron.BasisTypes.SIMPLEX
    with pytest.raises(iron.CMFEError):
        b.CreateFinish()
    cs = iron.CoordinateSystem()
    cs.CreateStart(1)
    cs.DimensionSet(2)
    with pytest.raises(iron.CMFEError):
        cs.CreateFinish()
    es = iron.EquationsSet()
    with pytest.raises(iron.CMFEError, match="outside the covered subset"):
        es.CreateStart(1, iron.Region(), iron.Field(), [iron.EquationsSetClasses.CLASSICAL_FIELD, 9, 1], 2,
                       iron.Field())
    d = iron.Decomposition()
    d.CreateStart(1, iron.Mesh())
    d.numberOfDomains = 4
    with pytest.raises(iron.CMFEError, match="one domain"):
        d.CreateFinish()
    eq = iron.Equations()
    with pytest.raises(iron.CMFEError):
        eq.JacobianFiniteDifferenceStepSizeSet(1, iron.FieldVariableTypes.U, 0.0)
    with pytest.raises(iron.CMFEError):
        eq.LinearMatrixGet(1, iron.DistributedMatrix())
