"""The oracle's geometrically nonlinear HEX8 element (the Green-Lagrange branch
of StructuralElement3D::internal_residual, src/elasticity/solid_element_3d.cpp:
299-409, strain operator :1309-1463), pinned the way the reference pins its
structural elements (tests/element/structural/2D/quad4/
mast_quad4_linear_structural_extension_internal_jacobian.cpp:45-367 and the
6th-order central differences of tests/test_helpers.cpp:53-105): the tangent is
the derivative of the residual, the element reduces to the linear one for small
displacements, a finite rigid rotation gives no residual, and the tangent is
symmetric."""
import numpy as np
import pytest

import oracle as O


def element(distort=0.0, seed=0):
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float) * [1.0, 0.8, 1.3]
    X += distort * np.random.default_rng(seed).uniform(-1, 1, X.shape)
    return X


def var_blocked(disp):
    """(8, 3) nodal displacements -> var-blocked element vector (u0..u7, v0.., w0..)"""
    return np.ascontiguousarray(disp.T.reshape(24))


def fd_jacobian(X, E, nu, u, h=1e-4):
    """6th-order central differences of the residual (the reference's stencil)"""
    J = np.zeros((24, 24))
    c = {1: 3 / 4, 2: -3 / 20, 3: 1 / 60}
    for j in range(24):
        col = np.zeros(24)
        for k, w in c.items():
            up, um = u.copy(), u.copy()
            up[j] += k * h
            um[j] -= k * h
            col += w * (O.hex8_internal_gl(X, E, nu, up, want_K=False)[0] -
                        O.hex8_internal_gl(X, E, nu, um, want_K=False)[0])
        J[:, j] = col / h
    return J


@pytest.mark.parametrize("distort", [0.0, 0.1])
def test_tangent_is_the_residual_derivative(distort):
    X = element(distort)
    u = np.random.default_rng(1).normal(scale=0.05, size=24)  # finite strains
    f, K = O.hex8_internal_gl(X, 1.0, 0.3, u)
    J = fd_jacobian(X, 1.0, 0.3, u)
    assert np.abs(K - J).max() <= 1e-8 * np.abs(K).max()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()


def test_small_displacements_give_the_linear_element():
    X = element(0.1)
    u = np.random.default_rng(2).normal(scale=1e-8, size=24)
    f, K = O.hex8_internal_gl(X, 2.0, 0.25, u)
    fl, Kl = O.hex8_internal(X, 2.0, 0.25, u)
    assert np.abs(K - Kl).max() <= 1e-6 * np.abs(Kl).max()
    assert np.abs(f - fl).max() <= 1e-6 * np.abs(fl).max()
    assert np.abs(O.hex8_internal_gl(X, 2.0, 0.25, np.zeros(24))[1] - Kl).max() <= 1e-14 * np.abs(Kl).max()


def test_rigid_rotation_is_stress_free():
    X = element(0.05)
    t = np.deg2rad(35.0)
    R = np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1]])
    ax = np.array([1.0, 2.0, 0.5]) / np.linalg.norm([1.0, 2.0, 0.5])
    Kx = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R2 = np.eye(3) + np.sin(0.6) * Kx + (1 - np.cos(0.6)) * Kx @ Kx  # Rodrigues
    for Q in (R, R2 @ R):
        disp = X @ Q.T - X + np.array([0.3, -0.2, 0.1])  # rotation + translation
        f, _ = O.hex8_internal_gl(X, 1.0, 0.3, var_blocked(disp))
        assert np.abs(f).max() <= 1e-13
        # the linear element is not invariant under a finite rotation
        fl, _ = O.hex8_internal(X, 1.0, 0.3, var_blocked(disp))
        assert np.abs(fl).max() > 1e-2
