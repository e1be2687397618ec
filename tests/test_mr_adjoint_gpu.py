"""Consistent tangent and hand-written adjoint (K6) of the Mooney-Rivlin residual.

Checked against central finite differences of the oracle's residual (step 1e-6 scaled, tolerance
1e-6 relative) and against Iron's one-sided finite-difference Jacobian
(src/equations_set_routines.F90:2839-2962; delta = (1 + ||dep||_2) * 1e-6, tolerance 1e-4 relative,
the truncation error of a one-sided difference).
"""
import numpy as np
import pytest
import torch

import oracle
from iron_gb300.elasticity import MooneyRivlinAssembly, mr_residual

pytestmark = pytest.mark.gpu

C1, C2 = 2.0, 6.0


def _state(A, seed, amp=0.02, p=-1.0):
    rng = np.random.default_rng(seed)
    x = A.xg.cpu().numpy()
    lam = 1.08
    z = x * np.array([lam, lam ** -0.5, lam ** -0.5])[:, None]
    z = z + rng.normal(0, amp / A.mesh.nelem[0], z.shape)
    return np.r_[z.ravel(), p + rng.normal(0, 0.2, A.n_lin)]


def _element(A, dep, e):
    x = A.xg.cpu().numpy()
    nq = A.n_q2
    en = A.mesh.elem_nodes[e]
    el = A.elin.cpu().numpy()[e]
    return x[:, en], dep[: 3 * nq].reshape(3, nq)[:, en], dep[3 * nq:][el]


def _central_fd(xe, ze, pe, h=1e-6):
    v = np.r_[ze.ravel(), pe]
    K = np.zeros((89, 89))
    for j in range(89):
        a, b = v.copy(), v.copy()
        a[j] += h
        b[j] -= h
        K[:, j] = (oracle.mr_element_residual(xe, a[:81].reshape(3, 27), a[81:], C1, C2)
                   - oracle.mr_element_residual(xe, b[:81].reshape(3, 27), b[81:], C1, C2)) / (2 * h)
    return K


def test_element_tangent_vs_finite_differences(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 1, 1), build_jacobian=False)
    dep = _state(A, 0)
    K = A.element_tangents(torch.from_numpy(dep).cuda(), [C1, C2]).cpu().numpy()
    delta = (1.0 + np.linalg.norm(dep)) * 1e-6
    for e in range(A.n_elements):
        xe, ze, pe = _element(A, dep, e)
        Kc = _central_fd(xe, ze, pe)
        scale = np.abs(Kc).max()
        assert np.abs(K[e] - Kc).max() <= 1e-6 * scale
        Kf = oracle.mr_element_jacobian_fd(xe, ze, pe, C1, C2, delta)
        assert np.abs(K[e] - Kf).max() <= 1e-4 * scale
        assert np.all(K[e][81:, 81:] == 0.0)


def test_assembled_tangent_times_vector_vs_residual_difference(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((3, 2, 2))
    dep = torch.from_numpy(_state(A, 1)).cuda()
    A.tangent(dep, [C1, C2])
    rp, ci, vals = A.to_iron_csr()
    rng = np.random.default_rng(2)
    d = rng.normal(0, 1, A.ndof)
    Kd = oracle.spmv(rp, ci, vals, d)
    h = 1e-6
    Rp = A.residual(dep + h * torch.from_numpy(d).cuda(), [C1, C2]).cpu().numpy()
    Rm = A.residual(dep - h * torch.from_numpy(d).cuda(), [C1, C2]).cpu().numpy()
    fd = (Rp - Rm) / (2 * h)
    assert np.abs(Kd - fd).max() <= 1e-6 * np.abs(fd).max()


def test_vjp_matches_transpose_tangent_and_parameter_fd(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 2))
    B = 3
    rng = np.random.default_rng(4)
    deps = np.stack([_state(A, s) for s in range(B)])
    cs = np.exp(rng.uniform(np.log(0.5), np.log(10.0), (B, 2)))
    v = rng.normal(0, 1, (B, A.ndof))
    du, dc = A.residual_vjp(torch.from_numpy(deps).cuda(), torch.from_numpy(cs).cuda(), torch.from_numpy(v).cuda())
    du, dc = du.cpu().numpy(), dc.cpu().numpy()
    for b in range(B):
        A.tangent(torch.from_numpy(deps[b]).cuda(), cs[b])
        rp, ci, vals = A.to_iron_csr()
        n = A.ndof
        KT_v = np.zeros(n)
        rows = np.repeat(np.arange(n), np.diff(rp))
        np.add.at(KT_v, ci - 1, vals * v[b][rows])
        assert np.abs(du[b] - KT_v).max() <= 1e-10 * np.abs(KT_v).max()
        for q in range(2):
            h = 1e-6 * cs[b, q]
            cp, cm = cs[b].copy(), cs[b].copy()
            cp[q] += h
            cm[q] -= h
            Rp = A.residual(torch.from_numpy(deps[b]).cuda(), cp).cpu().numpy()
            Rm = A.residual(torch.from_numpy(deps[b]).cuda(), cm).cpu().numpy()
            fd = v[b] @ (Rp - Rm) / (2 * h)
            assert abs(dc[b, q] - fd) <= 1e-7 * max(abs(fd), 1e-12) + 1e-9


def test_autograd_function(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 1, 1), build_jacobian=False)
    dep = torch.from_numpy(_state(A, 5)).cuda().requires_grad_(True)
    c = torch.tensor([C1, C2], dtype=torch.float64, device="cuda", requires_grad=True)
    R = mr_residual(A, dep, c)
    w = torch.randn_like(R)
    (R * w).sum().backward()
    du, dc = A.residual_vjp(dep.detach(), c.detach(), w)
    assert torch.allclose(dep.grad, du.reshape(-1), rtol=0, atol=1e-12 * du.abs().max().item())
    assert torch.allclose(c.grad, dc.reshape(-1), rtol=1e-12, atol=0)


def test_vjp_at_config_size_sampled(gfe_cuda):
    """The 16^3 Q2/Q1 mesh with 64 parameter sets (c10, c01 log-uniform in [0.5, 10], nodal
    perturbations N(0, (0.01 h)^2)): for four sampled parameter sets du equals K^T v of the assembled
    consistent tangent within 1e-10 and dc central differences of the residual in (c10, c01) within
    1e-7, and every set's result is the same as when it is computed alone."""
    A = MooneyRivlinAssembly.from_regular_mesh((16, 16, 16))
    B = 64
    rng = np.random.default_rng(11)
    x = A.xg.cpu().numpy()
    h = 1.0 / 16
    deps = np.empty((B, A.ndof))
    for b in range(B):
        z = x + rng.normal(0, 0.01 * h, x.shape)
        deps[b] = np.r_[z.ravel(), rng.normal(0, 0.1, A.n_lin)]
    cs = np.exp(rng.uniform(np.log(0.5), np.log(10.0), (B, 2)))
    v = rng.normal(0, 1, (B, A.ndof))
    dd, cc, vv = (torch.from_numpy(a).cuda() for a in (deps, cs, v))
    du, dc = A.residual_vjp(dd, cc, vv)
    for b in (0, 17, 40, 63):
        A.tangent(dd[b], cc[b])
        rp, ci, vals = A.to_iron_csr()
        n = A.ndof
        KT_v = np.zeros(n)
        rows = np.repeat(np.arange(n), np.diff(rp))
        np.add.at(KT_v, ci - 1, vals * v[b][rows])
        got = du[b].cpu().numpy()
        assert np.abs(got - KT_v).max() <= 1e-10 * np.abs(KT_v).max(), b
        for q in range(2):
            hq = 1e-6 * cs[b, q]
            cp, cm = cs[b].copy(), cs[b].copy()
            cp[q] += hq
            cm[q] -= hq
            Rp = A.residual(dd[b], cp).cpu().numpy()
            Rm = A.residual(dd[b], cm).cpu().numpy()
            fd = v[b] @ (Rp - Rm) / (2 * hq)
            assert abs(dc[b, q].item() - fd) <= 1e-7 * abs(fd) + 1e-9, (b, q)
        du1, dc1 = A.residual_vjp(dd[b], cc[b], vv[b])
        assert torch.equal(du1.reshape(-1), du[b]) and torch.equal(dc1.reshape(-1), dc[b])
