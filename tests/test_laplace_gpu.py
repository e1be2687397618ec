"""Parity of the GPU Laplace path (K3 structure, K1+K2 assembly, K7 solve) with the oracle.

Tolerances: structure bit-exact; FP64 element matrices and assembled values within
1e-13 x max|K| (different but equally valid rounding order); mixed (FP32 element arithmetic,
FP64 accumulation) within 2e-6 x max|K|; solutions within 1e-10 relative of the oracle's
FP64 solve at rtol 1e-12.
"""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300 import mesh as M
from iron_gb300.laplace import LaplaceAssembly, csr_structure
from iron_gb300._lib import GfeError

pytestmark = pytest.mark.gpu


def _mesh(ne, seed=0, jitter=True):
    m = M.RegularMesh(ne)
    if jitter:
        m.jitter_interior(seed)
    return m


def _kappa(E, seed):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(0.1), np.log(10.0), E))


@pytest.mark.parametrize("ne", [(1, 1, 1), (2, 3, 1), (5, 4, 3), (8, 8, 8)])
def test_structure_bit_exact(gfe_cuda, ne):
    m = _mesh(ne)
    rp, ci = csr_structure(torch.from_numpy(m.elem_nodes).cuda(), m.n_nodes)
    orp, oci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    assert np.array_equal(rp.cpu().numpy(), orp)
    assert np.array_equal(ci.cpu().numpy(), oci)


def test_structure_q2p1_bit_exact(gfe_cuda):
    ne = (3, 2, 2)
    e2 = M.regular_elements(ne, 2)
    el, l2g = M.linear_component(e2, 2)
    nq = int(np.prod([2 * n + 1 for n in ne]))
    dofs = np.concatenate([e2, e2 + nq, e2 + 2 * nq, el + 3 * nq], axis=1)
    nd = 3 * nq + len(l2g)
    rp, ci = csr_structure(torch.from_numpy(dofs).cuda(), nd)
    orp, oci = oracle.csr_structure(dofs, nd)
    assert np.array_equal(rp.cpu().numpy(), orp)
    assert np.array_equal(ci.cpu().numpy(), oci)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 2e-6), ("mixed_df", 5e-13)])
def test_element_matrices(gfe_cuda, precision, tol):
    m = _mesh((4, 3, 5), seed=1)
    kap = _kappa(m.n_elements, 2)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    K = A.element_matrices(precision).cpu().numpy()
    for e in range(m.n_elements):
        Ko = oracle.laplace_element(3, [1, 1, 1], [2, 2, 2], m.coords[:, m.elem_nodes[e]], kap[e])
        assert np.abs(K[e] - Ko).max() <= tol * np.abs(Ko).max(), e


@pytest.mark.parametrize("ne,seed", [((8, 8, 8), 0), ((8, 8, 8), 3), ((7, 3, 5), 1), ((1, 1, 1), 2),
                                     ((33, 9, 40), 4)])
@pytest.mark.parametrize("with_kappa", [False, True])
@pytest.mark.parametrize("path", ["regular", "general"])
def test_assembly_fp64(gfe_cuda, ne, seed, with_kappa, path):
    m = _mesh(ne, seed)
    kap = _kappa(m.n_elements, seed + 10) if with_kappa else None
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    assert A.regular == tuple(ne)
    A.rhs.fill_(7.0)
    v = A.assemble("fp64", path=path).cpu().numpy()
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    ov, orhs = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kap, rp, ci)
    assert np.abs(v - ov).max() <= 1e-13 * np.abs(ov).max()
    assert torch.count_nonzero(A.rhs).item() == 0


@pytest.mark.parametrize("path", ["regular", "general"])
def test_assembly_mixed_df_is_fp64_accurate(gfe_cuda, path):
    """Float-float element arithmetic on the FP32 pipes matches the FP64 oracle to 5e-13."""
    m = _mesh((12, 10, 9), 5)
    kap = _kappa(m.n_elements, 6)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    v = A.assemble("mixed_df", path=path).cpu().numpy()
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    ov, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kap, rp, ci)
    assert np.abs(v - ov).max() <= 5e-13 * np.abs(ov).max()
    assert np.array_equal(A.values32.cpu().numpy(), v.astype(np.float32))


def test_regular_check_rejects_other_structures(gfe_cuda):
    m = _mesh((4, 3, 2), 0)
    perm = np.random.default_rng(0).permutation(m.n_elements)
    A = LaplaceAssembly(m.elem_nodes[perm], m.coords)
    assert A.regular is None
    import ctypes as C
    from iron_gb300 import _lib
    bad = C.c_int64(0)
    # the structure of a 4x3x2 mesh is not the one of a 3x4x2 mesh
    _lib.call("gfe_laplace_regular_check", 3, 4, 2, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), C.byref(bad),
              _lib.stream_handle())
    assert bad.value > 0
    with pytest.raises(GfeError):
        A.assemble("fp64", path="regular")


def test_assembly_mixed_and_fp32_copy(gfe_cuda):
    m = _mesh((8, 8, 8), 0)
    kap = _kappa(m.n_elements, 5)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    v = A.assemble("mixed").cpu().numpy()
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    ov, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kap, rp, ci)
    scale = np.abs(ov).max()
    assert np.abs(v - ov).max() <= 2e-6 * scale
    v32 = A.values32.cpu().numpy()
    assert np.array_equal(v32, v.astype(np.float32))


def test_assembly_deterministic(gfe_cuda):
    m = _mesh((9, 7, 6), 4)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=_kappa(m.n_elements, 1))
    for path in ("regular", "general"):
        for prec in ("fp64", "mixed_df"):
            a = A.assemble(prec, path=path).clone()
            b = A.assemble(prec, path=path).clone()
            assert torch.equal(a, b)


def test_greedy_colouring_permuted_mesh(gfe_cuda):
    """General (unstructured) path: elements in random order, greedy colouring."""
    m = _mesh((5, 4, 4), 2)
    perm = np.random.default_rng(0).permutation(m.n_elements)
    en = m.elem_nodes[perm]
    A = LaplaceAssembly(en, m.coords)
    v = A.assemble("fp64").cpu().numpy()
    rp, ci = oracle.csr_structure(en, m.n_nodes)
    ov, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], en, m.coords, None, rp, ci)
    assert np.abs(v - ov).max() <= 1e-13 * np.abs(ov).max()


def test_missing_slot_reported(gfe_cuda):
    """A structure lacking entries is an error (MATRIX_VALUES_ADD_DP2 flags absent columns)."""
    m = _mesh((3, 3, 3), 0)
    # structure of a different connectivity: diagonal-only rows
    N = m.n_nodes
    rp = torch.arange(1, N + 2, dtype=torch.int32, device="cuda")
    ci = torch.arange(1, N + 1, dtype=torch.int32, device="cuda")
    order, ptr = m.colouring()
    A = LaplaceAssembly(m.elem_nodes, m.coords, colour_elems=order, colour_ptr=ptr, structure=(rp, ci))
    with pytest.raises(GfeError):
        A.assemble("fp64")


def _cfg1_bcs(m):
    x0 = np.zeros(m.n_nodes)
    fixed = np.zeros(m.n_nodes, np.uint8)
    left, right = m.face_nodes(0, 0), m.face_nodes(0, 1)
    fixed[left] = 1
    fixed[right] = 1
    x0[right] = 1.0
    return fixed, x0


@pytest.mark.parametrize("seed", [0, 1, 2, 3, 4])
def test_config1_solve_vs_oracle(gfe_cuda, seed):
    """Config 1: 8^3 jittered unit cube, u = 0 at x = 0, u = 1 at x = 1 -> patch test u = x."""
    m = _mesh((8, 8, 8), seed)
    A = LaplaceAssembly.from_regular_mesh(m)
    A.assemble("fp64")
    fixed, x0 = _cfg1_bcs(m)
    x = torch.from_numpy(x0).cuda()
    info = A.solve(torch.from_numpy(fixed).cuda(), x, rtol=1e-12)
    assert info.relative_residual <= 1e-12
    u = x.cpu().numpy()
    assert np.abs(u - m.coords[0]).max() < 1e-10
    rp, ci, vals = A.to_iron_csr()
    uo, _, _ = oracle.cg_dirichlet(rp, ci, vals, None, fixed, x0, rtol=1e-13)
    assert np.abs(u - uo).max() <= 1e-10 * np.abs(uo).max()


def test_kappa_solve_fp64_and_mixed(gfe_cuda):
    """Config-2-type problem (log-uniform conductivity) on a small mesh: both precisions reach
    the FP64 oracle solution to 1e-10 relative when the residual is formed with the FP64 matrix."""
    m = _mesh((10, 9, 8), 7)
    kap = _kappa(m.n_elements, 8)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    A.assemble("fp64")
    fixed, x0 = _cfg1_bcs(m)
    rp, ci, vals = A.to_iron_csr()
    uo, _, _ = oracle.cg_dirichlet(rp, ci, vals, None, fixed, x0, rtol=1e-14)
    x = torch.from_numpy(x0).cuda()
    info = A.solve(torch.from_numpy(fixed).cuda(), x, rtol=1e-12, precision="fp64")
    assert np.abs(x.cpu().numpy() - uo).max() <= 1e-10 * np.abs(uo).max(), info
    A.values32 = A.values.float()
    x2 = torch.from_numpy(x0).cuda()
    info2 = A.solve(torch.from_numpy(fixed).cuda(), x2, rtol=1e-12, precision="mixed")
    assert info2.relative_residual <= 1e-12
    assert np.abs(x2.cpu().numpy() - uo).max() <= 1e-10 * np.abs(uo).max(), info2


@pytest.mark.parametrize("precision,slab_layers", [("mixed_df", 8), ("mixed", 24), ("fp64", 16), ("mixed_df", 16),
                                                   ("mixed_df", 64)])
def test_slab_pipelined_host_assembly_equals_device(gfe_cuda, precision, slab_layers):
    """gfe_laplace_assemble_regular_host (inputs uploaded and converted slab by slab, device-to-host
    copies overlapping later slabs) gives exactly the values of the one-shot regular-mesh assembly;
    the device copies of the inputs are cleared first, so every layer a slab reads must have been
    uploaded before it runs, and every CSR entry must come back."""
    m = _mesh((9, 7, 21), 5)
    kap = _kappa(m.n_elements, 6)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    ref = A.assemble(precision, path="regular").cpu().clone()
    host = torch.full((A.nnz,), float("nan"), dtype=torch.float64).pin_memory()
    A.values.zero_()
    A.coords.zero_()
    A.kappa.zero_()
    coords_h = torch.from_numpy(m.coords).pin_memory()
    kappa_h = torch.from_numpy(kap).pin_memory()
    A.assemble_to_host(host, precision, coords_host=coords_h, kappa_host=kappa_h, slab_layers=slab_layers)
    torch.cuda.synchronize()
    assert torch.equal(host, ref)
    # inputs already resident: the device copies are used as they are
    host2 = torch.zeros(A.nnz, dtype=torch.float64).pin_memory()
    A.assemble_to_host(host2, precision, slab_layers=slab_layers)
    torch.cuda.synchronize()
    assert torch.equal(host2, ref)


def test_host_pipeline_rejects_bad_arguments(gfe_cuda):
    m = _mesh((3, 3, 3), 1)
    A = LaplaceAssembly.from_regular_mesh(m)
    host = torch.zeros(A.nnz, dtype=torch.float64)
    with pytest.raises(GfeError, match="multiple of 8"):
        A.assemble_to_host(host, "mixed_df", slab_layers=12)
    with pytest.raises(GfeError, match="coords_host"):
        A.assemble_to_host(host, "mixed_df", coords_host=torch.zeros(5, dtype=torch.float64))
