"""Parity of the GPU Mooney-Rivlin residual (K4) and Iron-analytic Jacobian (K5) with the oracle.

Tolerances (FP64 on both sides, different summation order): residual within 1e-12 x max|R_ref|
(undeformed-scale forces), Jacobian within 1e-12 x max|K|; CSR structure bit-exact.
"""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300.elasticity import MooneyRivlinAssembly

pytestmark = pytest.mark.gpu

C1, C2 = 2.0, 6.0


def _state(A, seed, amp=0.02, p=-1.0):
    rng = np.random.default_rng(seed)
    x = A.xg.cpu().numpy()
    lam = 1.05
    z = x * np.array([lam, lam ** -0.5, lam ** -0.5])[:, None]
    z = z + rng.normal(0, amp / A.mesh.nelem[0], z.shape)
    pr = p + rng.normal(0, 0.2, A.n_lin)
    return np.r_[z.ravel(), pr]


@pytest.mark.parametrize("ne", [(1, 1, 1), (2, 3, 2), (4, 4, 4)])
def test_residual_matches_oracle(gfe_cuda, ne):
    A = MooneyRivlinAssembly.from_regular_mesh(ne, build_jacobian=False)
    dep = _state(A, 0)
    R = A.residual(torch.from_numpy(dep).cuda(), [C1, C2]).cpu().numpy()
    Ro = oracle.mr_assemble_residual(A.mesh.elem_nodes, A.elin.cpu().numpy(), A.n_q2, A.n_lin,
                                     A.xg.cpu().numpy(), dep, [C1, C2])
    assert np.abs(R - Ro).max() <= 1e-12 * np.abs(Ro).max()


def test_residual_batched_parameter_sets(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((3, 2, 2), build_jacobian=False)
    B = 5
    rng = np.random.default_rng(3)
    deps = np.stack([_state(A, s) for s in range(B)])
    cs = np.exp(rng.uniform(np.log(0.5), np.log(10.0), (B, 2)))
    R = A.residual(torch.from_numpy(deps).cuda(), torch.from_numpy(cs)).cpu().numpy()
    for b in range(B):
        Ro = oracle.mr_assemble_residual(A.mesh.elem_nodes, A.elin.cpu().numpy(), A.n_q2, A.n_lin,
                                         A.xg.cpu().numpy(), deps[b], cs[b])
        assert np.abs(R[b] - Ro).max() <= 1e-12 * np.abs(Ro).max()
    # each result is the same alone and in the batch
    R1 = A.residual(torch.from_numpy(deps[2]).cuda(), torch.from_numpy(cs[2])).cpu().numpy()
    assert np.array_equal(R1, R[2])


def test_undeformed_residual_zero(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((3, 3, 3), build_jacobian=False)
    R = A.residual(A.initial_state(0.0), [C1, C2]).cpu().numpy()
    assert np.abs(R).max() < 1e-13


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5), ("tf32x3", 2e-5), ("tf32", 4e-3)])
def test_element_jacobians_match_oracle(gfe_cuda, precision, tol):
    """Iron's analytic element Jacobian; 'mixed' = FP32 kinematics (FP64 volume Jacobians) and FP32 basis-gradient contraction,
    'tf32x3' / 'tf32' = the contraction on the tensor cores (three-pass split / one TF32 pass);
    tolerances relative to max|K|."""
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 1), build_jacobian=False)
    dep = _state(A, 1)
    K = A.element_jacobians(torch.from_numpy(dep).cuda(), [C1, C2], precision=precision).cpu().numpy()
    x = A.xg.cpu().numpy()
    nq = A.n_q2
    el = A.elin.cpu().numpy()
    for e in range(A.n_elements):
        en = A.mesh.elem_nodes[e]
        Ko = oracle.mr_element_jacobian(x[:, en], dep[: 3 * nq].reshape(3, nq)[:, en], dep[3 * nq:][el[e]], C1, C2)
        assert np.abs(K[e] - Ko).max() <= tol * np.abs(Ko).max(), e


@pytest.mark.parametrize("ne", [(1, 1, 1), (3, 2, 2)])
def test_assembled_jacobian_matches_oracle(gfe_cuda, ne):
    A = MooneyRivlinAssembly.from_regular_mesh(ne)
    dep = _state(A, 2)
    v = A.jacobian(torch.from_numpy(dep).cuda(), [C1, C2]).cpu().numpy()
    rp, ci, _ = A.to_iron_csr()
    elem_dofs = A.elem_dofs.cpu().numpy()
    orp, oci = oracle.csr_structure(elem_dofs, A.ndof)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    vo = oracle.mr_assemble_jacobian(A.mesh.elem_nodes, A.elin.cpu().numpy(), A.n_q2, A.n_lin, A.xg.cpu().numpy(),
                                     dep, [C1, C2], orp, oci)
    assert np.abs(v - vo).max() <= 1e-12 * np.abs(vo).max()


def test_slot_map_beyond_2pow30_entries(gfe_cuda):
    """59^3 Q2/Q1 mesh: the Jacobian has more than 2^30 non-zeros, so the bisection midpoint of
    rows near the end would overflow int32 if computed as (lo + hi) / 2.  Sampled slot-map entries
    (indexed by element number) of the last elements in colour order point at their (row, column)
    in the CSR."""
    A = MooneyRivlinAssembly.from_regular_mesh((59, 59, 59))
    assert A.nnz > 2 ** 30
    torch.cuda.synchronize()
    rp = A.row_ptr
    ce = A.colour_elems
    dofs = A.elem_dofs
    for item in (A.n_elements - 1, A.n_elements - 2, A.colour_ptr[-2]):
        e = int(ce[item])
        d = dofs[e].cpu().numpy()
        sl = A.slots[e].cpu().numpy()
        for r in (0, 40, 80, 81, 88):
            lo, hi = int(rp[d[r]]) - 1, int(rp[d[r] + 1]) - 1
            cols = A.col_idx[lo:hi].cpu().numpy()
            for c in range(89):
                if r >= 81 and c >= 81:
                    continue
                pos = lo + int(np.searchsorted(cols, d[c] + 1))
                assert sl[r, c] == pos, (item, r, c)
    del A
    torch.cuda.empty_cache()


@pytest.mark.parametrize("precision,tol", [("mixed", 2e-5), ("tf32x3", 2e-5), ("tf32", 4e-3)])
def test_tensor_core_assembly_matches_fp64(gfe_cuda, precision, tol):
    """CSR assembly (element matrices, then the row gather) of the analytic Jacobian and the
    consistent tangent with the FP32 CUDA-core and the tensor-core contractions against the FP64
    contraction; the FP64 element matrices widened from each path's give the same CSR values
    through the oracle's scatter."""
    A = MooneyRivlinAssembly.from_regular_mesh((5, 4, 3))
    dep = torch.from_numpy(_state(A, 4)).cuda()
    slots = A.slots.cpu().numpy().reshape(A.n_elements, -1)
    for fn, dense in (("jacobian", "element_jacobians"), ("tangent", "element_tangents")):
        ref = getattr(A, fn)(dep, [C1, C2], precision="fp64").clone()
        got = getattr(A, fn)(dep, [C1, C2], precision=precision).cpu().numpy()
        assert np.abs(got - ref.cpu().numpy()).max() <= tol * ref.abs().max().item(), fn
        # the row gather sums exactly the FP32 element matrices of this precision: in FP32, in
        # ascending element order (np.add.at takes the entries element by element), widened to FP64
        K = getattr(A, dense)(dep, [C1, C2], precision=precision).cpu().numpy().reshape(A.n_elements, -1)
        keep = slots >= 0
        keep &= ~((np.arange(89 * 89) // 89 >= 81) & (np.arange(89 * 89) % 89 >= 81))[None, :]
        K32 = K[keep].astype(np.float32)
        assert np.array_equal(K32.astype(np.float64), K[keep]), fn
        v = np.zeros(A.nnz, np.float32)
        np.add.at(v, slots[keep], K32)
        assert np.array_equal(got, v.astype(np.float64)), fn


@pytest.mark.parametrize("ne", [(1, 1, 1), (2, 3, 1), (3, 2, 4), (5, 1, 2)])
def test_closed_form_structure_equals_sorted_structure(gfe_cuda, ne):
    """gfe_mr_regular_structure (boxes of the regular Q2/Q1 mesh) is bit-identical to the structure
    sorted and deduplicated from the element DOF lists (gfe_csr_structure)."""
    from iron_gb300.laplace import csr_structure
    A = MooneyRivlinAssembly.from_regular_mesh(ne)
    assert A.regular == ne
    rp, ci = csr_structure(A.elem_dofs, A.ndof)
    assert torch.equal(A.row_ptr, rp) and torch.equal(A.col_idx, ci)
