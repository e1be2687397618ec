"""Generalised Laplace on the GPU (gfe_laplace_assemble_generalised): a full conductivity tensor per
element in a material frame, against the oracle's restatement of Iron's generalised element
(src/Laplace_equations_routines.F90:585-707, src/coordinate_routines.F90:3841-4127) on jittered
meshes, with nodal fibre fields of one to three angles and without one; CSR values within
1e-13 x max|K|.  An isotropic tensor gives the standard assembly, and a non-finite conductivity
sets the device error word."""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300._lib import GfeError
from iron_gb300.laplace import LaplaceAssembly
from iron_gb300.mesh import RegularMesh

pytestmark = pytest.mark.gpu


def _problem(nelem, seed):
    m = RegularMesh(nelem)
    m.jitter_interior(seed)
    rng = np.random.default_rng(seed)
    E = m.n_elements
    # symmetric positive definite tensors: L L^T + 0.2 I with log-uniform scaling
    L = rng.normal(size=(E, 3, 3))
    T = L @ L.transpose(0, 2, 1) + 0.2 * np.eye(3)
    T *= np.exp(rng.uniform(np.log(0.1), np.log(10.0), E))[:, None, None]
    cond = np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], T[:, 0, 1], T[:, 1, 2], T[:, 0, 2]])
    return m, cond, rng


@pytest.mark.parametrize("n_angles", [0, 1, 2, 3])
def test_generalised_assembly_matches_oracle(gfe_cuda, n_angles):
    m, cond, rng = _problem((5, 4, 3), 7 + n_angles)
    fibre = rng.uniform(-1.2, 1.2, (n_angles, m.n_nodes)) if n_angles else None
    A = LaplaceAssembly.from_regular_mesh(m, device=gfe_cuda)
    v = A.assemble_generalised(cond, fibre).cpu().numpy()
    rp, ci = A.row_ptr.cpu().numpy(), A.col_idx.cpu().numpy()
    ov, orhs = oracle.laplace_generalised_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, cond.T.copy(),
                                                   rp, ci, fibre)
    assert np.abs(v - ov).max() <= 1e-13 * np.abs(ov).max()
    assert np.all(A.rhs.cpu().numpy() == 0.0)
    # rows of a pure-Neumann Laplacian sum to zero
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    assert np.abs(np.bincount(rows, weights=v)).max() <= 1e-12 * np.abs(v).max()


def test_isotropic_tensor_equals_standard_assembly(gfe_cuda):
    m, _, rng = _problem((4, 4, 4), 3)
    kap = np.exp(rng.uniform(np.log(0.1), np.log(10.0), m.n_elements))
    cond = np.vstack([kap, kap, kap, 0 * kap, 0 * kap, 0 * kap])
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap, device=gfe_cuda)
    std = A.assemble("fp64", path="general").clone()
    gen = A.assemble_generalised(cond, rng.uniform(-1, 1, (3, m.n_nodes)))
    assert (torch.abs(gen - std).max() <= 1e-13 * torch.abs(std).max()).item()


def test_non_finite_conductivity_is_reported(gfe_cuda):
    m, cond, _ = _problem((3, 3, 3), 1)
    cond[4, 5] = np.nan
    A = LaplaceAssembly.from_regular_mesh(m, device=gfe_cuda)
    with pytest.raises(GfeError, match="non-finite"):
        A.assemble_generalised(cond)
    # the error word was cleared: a good assembly afterwards succeeds
    cond[4, 5] = 0.1
    A.assemble_generalised(cond)


def test_argument_checks(gfe_cuda):
    m, cond, _ = _problem((2, 2, 2), 1)
    A = LaplaceAssembly.from_regular_mesh(m, device=gfe_cuda)
    with pytest.raises(GfeError):
        A.assemble_generalised(cond[:5])
    with pytest.raises(GfeError):
        A.assemble_generalised(cond, np.zeros((4, m.n_nodes)))
    with pytest.raises(GfeError):
        A.assemble_generalised(cond, np.zeros((2, m.n_nodes + 1)))
