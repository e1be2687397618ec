"""The oracle's generalised Laplace element (full conductivity tensor in a material frame,
src/Laplace_equations_routines.F90:585-707 with src/coordinate_routines.F90:3841-4127) against
known answers: an isotropic tensor reduces to the standard element with any fibre field; an
axis-aligned box with a diagonal tensor is the standard element of the box stretched by
1/sqrt(k_i), times sqrt(k1 k2 k3); on a cube, fibre, imbrication and sheet angles act as the
rotation F = Rz(a) Ry(b) Rx(c) of the tensor, C = F^T K F."""
import numpy as np
import pytest

import oracle

TRI = ([1, 1, 1], [2, 2, 2])
CORNERS = np.array([[0, 1, 0, 1, 0, 1, 0, 1], [0, 0, 1, 1, 0, 0, 1, 1], [0, 0, 0, 0, 1, 1, 1, 1]], float)


def _gen(x, k6, fibre=None):
    return oracle.laplace_generalised_element(3, *TRI, x, k6, fibre)


def _std(x, kappa=1.0):
    return oracle.laplace_element(3, *TRI, x, kappa)


def _tensor(k6):
    k = np.diag(k6[:3]).astype(float)
    k[0, 1] = k[1, 0] = k6[3]
    k[1, 2] = k[2, 1] = k6[4]
    k[0, 2] = k[2, 0] = k6[5]
    return k


def _k6(K):
    return [K[0, 0], K[1, 1], K[2, 2], K[0, 1], K[1, 2], K[0, 2]]


@pytest.mark.parametrize("fibre", [None, 1, 3])
def test_isotropic_tensor_is_the_standard_element(fibre):
    rng = np.random.default_rng(3)
    x = CORNERS + rng.uniform(-0.15, 0.15, (3, 8))
    f = None if fibre is None else rng.uniform(-1.0, 1.0, (fibre, 8))
    K = _gen(x, [2.5, 2.5, 2.5, 0.0, 0.0, 0.0], f)
    Ks = _std(x, 2.5)
    assert np.abs(K - Ks).max() <= 1e-14 * np.abs(Ks).max()


def test_axis_aligned_box_with_diagonal_tensor():
    h = np.array([0.7, 1.3, 0.4])
    k = np.array([3.0, 0.5, 1.7])
    K = _gen(CORNERS * h[:, None], [*k, 0.0, 0.0, 0.0])
    Ks = np.sqrt(k.prod()) * _std(CORNERS * (h / np.sqrt(k))[:, None])
    assert np.abs(K - Ks).max() <= 1e-13 * np.abs(Ks).max()


@pytest.mark.parametrize("angles", [[0.4], [0.4, -0.3], [0.4, -0.3, 1.1]])
def test_fibre_angles_rotate_the_tensor_on_a_cube(angles):
    rng = np.random.default_rng(5)
    A = rng.normal(size=(3, 3))
    Km = A @ A.T + 0.5 * np.eye(3)
    a = list(angles) + [0.0] * (3 - len(angles))
    ca, sa, cb, sb, cg, sg = np.cos(a[0]), np.sin(a[0]), np.cos(a[1]), np.sin(a[1]), np.cos(a[2]), np.sin(a[2])
    Rz = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    Ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    Rx = np.array([[1, 0, 0], [0, cg, -sg], [0, sg, cg]])
    F = Rz @ Ry @ Rx
    x = CORNERS * 0.8
    fib = np.repeat(np.array(angles, float)[:, None], 8, axis=1)  # constant over the element
    K = _gen(x, _k6(Km), fib)
    Kr = _gen(x, _k6(F.T @ Km @ F))
    assert np.abs(K - Kr).max() <= 1e-13 * np.abs(Kr).max()
    # a rotated anisotropic tensor gives a different (and unsymmetric on a distorted element) matrix
    assert np.abs(K - _gen(x, _k6(Km))).max() > 1e-3 * np.abs(K).max()


def test_rows_sum_to_zero_and_distorted_elements_are_unsymmetric():
    rng = np.random.default_rng(9)
    x = CORNERS + rng.uniform(-0.15, 0.15, (3, 8))
    K = _gen(x, [2.0, 1.0, 0.5, 0.3, -0.2, 0.1], rng.uniform(-1, 1, (3, 8)))
    assert np.abs(K.sum(axis=1)).max() <= 1e-14 * np.abs(K).max()
    assert np.abs(K - K.T).max() > 1e-3 * np.abs(K).max()


def test_two_dimensional_isotropic_reduces_to_standard():
    rng = np.random.default_rng(2)
    x = np.array([[0, 1, 0, 1], [0, 0, 1, 1]], float) + rng.uniform(-0.1, 0.1, (2, 4))
    K = oracle.laplace_generalised_element(2, [1, 1], [2, 2], x, [1.5, 1.5, 0.0], rng.uniform(-1, 1, (1, 4)))
    Ks = oracle.laplace_element(2, [1, 1], [2, 2], x, 1.5)
    assert np.abs(K - Ks).max() <= 1e-14 * np.abs(Ks).max()
