"""Known-answer checks of the oracle's Mooney-Rivlin (MOONEY_RIVLIN_SUBTYPE) restatement (CPU only).

Iron ships no MR golden vector that matches this source revision (the Cantilever fixture shows a
gravity sag that the MR residual branch has commented out), so the restatement is pinned by
derivations: zero residual in the undeformed state, the homogeneous incompressible uniaxial
stretch with traction-free lateral faces, Iron-style one-sided finite differences against central
differences, and the p-u block of Iron's analytic Jacobian against finite differences.
"""
import numpy as np

import oracle

C1, C2 = 2.0, 6.0  # c10, c01 of tests/FiniteElasticity/Cantilever.F90:356-357


def _unit_element(h=1.0):
    en = oracle.regular_mesh([1, 1, 1], 2)
    x = oracle.regular_coords([1, 1, 1], 2, [0, 0, 0], [h, h, h])
    return np.ascontiguousarray(x[:, en[0]])


def _stretch(xe, lam):
    z = xe.copy()
    z[0] *= lam
    z[1] *= lam ** -0.5
    z[2] *= lam ** -0.5
    return z


def _traction_free_pressure(lam):
    F = np.diag([lam, lam ** -0.5, lam ** -0.5])
    Cb = F.T @ F
    S = -2 * C2 * Cb + 2 * (C1 + np.trace(Cb) * C2) * np.eye(3)
    sb = F @ S @ F.T
    return np.trace(sb) / 3 - sb[1, 1], sb[0, 0] - sb[1, 1]


def test_undeformed_state_has_zero_residual():
    xe = _unit_element(0.5)
    R = oracle.mr_element_residual(xe, xe, np.zeros(8), C1, C2)
    assert np.abs(R).max() < 1e-14


def test_uniaxial_stretch_traction_free():
    """F = diag(l, l^-1/2, l^-1/2) (J = 1): with p chosen so sigma_22 = sigma_33 = 0 the lateral
    nodal forces vanish, the pressure rows vanish (J - 1 = 0), and the axial forces integrate to
    sigma_11 times the face area."""
    xe = _unit_element(1.0)
    for lam in (1.02, 1.1, 0.9):
        p, s11 = _traction_free_pressure(lam)
        R = oracle.mr_element_residual(xe, _stretch(xe, lam), np.full(8, p), C1, C2)
        assert np.abs(R[27:81]).max() < 1e-12
        assert np.abs(R[81:]).max() < 1e-14
        # axial nodal forces on the face x = l sum to sigma_11 * deformed face area (lam^-1)
        face = [ns for ns in range(27) if ns % 3 == 2]
        assert abs(R[face].sum() - s11 * lam ** -1.0) < 1e-11 * abs(s11)


def test_fd_jacobian_iron_style_matches_central_differences():
    xe = _unit_element(1.0)
    rng = np.random.default_rng(0)
    p, _ = _traction_free_pressure(1.1)
    z = _stretch(xe, 1.1) + rng.normal(0, 0.01, (3, 27))
    pe = np.full(8, p) + rng.normal(0, 0.1, 8)
    v = np.r_[z.ravel(), pe]
    delta = (1.0 + np.linalg.norm(v)) * 1e-6  # src/equations_set_routines.F90:2902-2904
    Kf = oracle.mr_element_jacobian_fd(xe, z, pe, C1, C2, delta)
    h = 1e-5
    Kc = np.zeros((89, 89))
    for j in range(89):
        a, b = v.copy(), v.copy()
        a[j] += h
        b[j] -= h
        Kc[:, j] = (oracle.mr_element_residual(xe, a[:81].reshape(3, 27), a[81:], C1, C2)
                    - oracle.mr_element_residual(xe, b[:81].reshape(3, 27), b[81:], C1, C2)) / (2 * h)
    assert np.abs(Kf - Kc).max() <= 1e-4 * np.abs(Kc).max()
    # Iron's analytic tangent: its p-u block is the exact derivative of the pressure rows ...
    Ka = oracle.mr_element_jacobian(xe, z, pe, C1, C2)
    assert np.abs(Ka[81:, :81] - Kc[81:, :81]).max() <= 1e-8 * np.abs(Kc[81:, :81]).max()
    # ... its u-u block is symmetric (lower triangle mirrored) and not the exact derivative of
    # Iron's deviatoric residual (Iron flags it "not validated", finite_elasticity_routines.F90:737)
    assert np.array_equal(Ka[:81, :81], Ka[:81, :81].T)
    assert np.abs(Ka[:81, :81] - Kc[:81, :81]).max() > 1e-2 * np.abs(Kc[:81, :81]).max()


def test_assembled_residual_equals_sum_of_elements():
    ne = (2, 1, 1)
    e2 = oracle.regular_mesh(ne, 2)
    el, l2g = oracle.linear_component(e2, (3, 3, 3))
    x = oracle.regular_coords(ne, 2, [0, 0, 0], [2.0, 1.0, 1.0])
    nq, nl = x.shape[1], len(l2g)
    rng = np.random.default_rng(1)
    dep = np.r_[(x + rng.normal(0, 0.01, x.shape)).ravel(), rng.normal(0, 0.5, nl)]
    R = oracle.mr_assemble_residual(e2, el, nq, nl, x, dep, [C1, C2])
    R2 = np.zeros_like(R)
    for e in range(2):
        xe = x[:, e2[e]]
        ze = dep[: 3 * nq].reshape(3, nq)[:, e2[e]]
        pe = dep[3 * nq:][el[e]]
        Re = oracle.mr_element_residual(xe, ze, pe, C1, C2)
        dofs = np.r_[e2[e], e2[e] + nq, e2[e] + 2 * nq, el[e] + 3 * nq]
        np.add.at(R2, dofs, Re)
    assert np.abs(R - R2).max() < 1e-13
