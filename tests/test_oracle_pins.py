"""The FP64 oracle against MAST's own known answers (CPU only).

Known-answer values come from tests/golden/reference_pins.json, extracted from
the reference's unit-test sources by tests/golden/make_reference_pins.py:
  - C matrices: tests/material/mast_isotropic_material.cpp:272-445, 611-708;
  - QUAD4 membrane element properties:
    tests/element/structural/2D/quad4/
    mast_quad4_linear_structural_extension_internal_jacobian.cpp:45-367
    (6th-order FD Jacobian with the reference's step and margin, symmetry,
    singularity, invariance to rigid motion and to the fixed displacement vector);
  - shape functions: mast_quad4_structural_shape_functions.cpp:62-101.
Paths without reference golden data (HEX8, heat element, assembly, solves,
sensitivities) are pinned by FD Jacobians, rigid-body modes, the patch test,
scipy direct solves, FD of the outputs and an analytic 1D conduction solution.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "reference_pins.json")))


def approx_equal(a, b, margin=0.0, eps=100 * np.finfo(np.float32).eps):
    """Catch::Approx semantics used by the reference tests."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    d = np.abs(a - b)
    return bool(np.all((d <= margin) | (d <= eps * np.maximum(np.abs(a), np.abs(b)))))


# ----------------------------------------------------------------- materials
def test_isotropic_3d_stiffness_matches_reference_truth():
    m = PINS["material"]
    C = O.iso_stiffness_3d(m["E"], m["nu"])
    T = np.array(m["C3d_true"])
    assert np.allclose(C, T, rtol=1e-13, atol=0)
    assert np.allclose(C, C.T) and np.all(np.linalg.eigvalsh(C) > 0)


@pytest.mark.parametrize("plane_stress,key", [(True, "C2d_plane_stress_true"),
                                              (False, "C2d_plane_strain_true")])
def test_isotropic_2d_stiffness_matches_reference_truth(plane_stress, key):
    m = PINS["material"]
    C = O.iso_stiffness_2d(m["E"], m["nu"], plane_stress)
    assert np.allclose(C, np.array(m[key]), rtol=1e-13, atol=0)


# ----------------------------------------------------------------- shape functions
def test_shape_functions_partition_of_unity_and_kronecker():
    rng = np.random.default_rng(0)
    for _ in range(20):
        xi = rng.uniform(-1, 1, 3)
        phi, dphi = np.zeros(8), np.zeros(24)
        O.lib().or_hex8_shape(xi, phi, dphi)
        assert abs(phi.sum() - 1) < 1e-14 and np.abs(dphi.reshape(8, 3).sum(0)).max() < 1e-14
        phi4, d4 = np.zeros(4), np.zeros(8)
        O.lib().or_quad4_shape(xi[:2].copy(), phi4, d4)
        assert abs(phi4.sum() - 1) < 1e-14
    corners = [(-1, -1), (1, -1), (1, 1), (-1, 1)]
    for a, c in enumerate(corners):
        phi4, d4 = np.zeros(4), np.zeros(8)
        O.lib().or_quad4_shape(np.array(c, float), phi4, d4)
        assert np.allclose(phi4, np.eye(4)[a])


# ----------------------------------------------------------------- QUAD4 membrane
def transform_element(X0, shift_x, shift_y, shift_z, scale_x, scale_y, rot_x, rot_y, rot_z,
                      shear_x=0.0, shear_y=0.0):
    """Same sequence as TEST::transform_element (tests/test_helpers.cpp:303-396)."""
    c = X0.mean(axis=1, keepdims=True)
    V = np.diag([scale_x, scale_y, 1.0]) @ (X0 - c)
    K = np.eye(3)
    K[0, 1], K[1, 0] = shear_x, shear_y
    V = K @ V
    t = np.radians(rot_z)
    Rz = np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1]])
    t = np.radians(rot_y)
    Ry = np.array([[np.cos(t), 0, -np.sin(t)], [0, 1, 0], [np.sin(t), 0, np.cos(t)]])
    t = np.radians(rot_x)
    Rx = np.array([[1, 0, 0], [0, np.cos(t), -np.sin(t)], [0, np.sin(t), np.cos(t)]])
    V = Rx @ (Ry @ (Rz @ V))
    return c + V + np.array([[shift_x], [shift_y], [shift_z]])


def fd_jacobian(resid, u0, delta):
    """6th-order central FD of TEST::approximate_internal_jacobian_with_finite_difference
    (tests/test_helpers.cpp:53-105)."""
    n = u0.shape[0]
    J = np.zeros((n, n))
    for i in range(n):
        def r(k):
            u = u0.copy()
            u[i] += k * delta
            return resid(u)
        J[:, i] = (-r(-3) + 9 * r(-2) - 45 * r(-1) + 45 * r(1) - 9 * r(2) + r(3)) / (60 * delta)
    return J


QP = PINS["quad4_membrane"]
X0 = np.array(QP["coords_3x4"]).reshape(3, 4)


def membrane(Xc, u=None):
    return O.quad4_membrane_internal(Xc[:2].T.copy(), QP["E"], QP["nu"], QP["thickness"], u)


def test_membrane_baseline_properties():
    f0, J0 = membrane(X0)
    margin = np.abs(J0).mean() * QP["margin_factor"]
    Jfd = fd_jacobian(lambda u: membrane(X0, u)[0], np.zeros(8), QP["fd_delta"])
    assert approx_equal(J0, Jfd, margin)
    assert approx_equal(J0, J0.T)
    w = np.linalg.eigvalsh(J0)
    assert np.sum(np.abs(w) < 1e-9 * np.abs(w).max()) == 3  # 2 translations + rotation
    # invariant to the fixed displacement vector of the reference test (u, v blocks)
    u = np.array(QP["elem_sol_24"][:8])
    f, J = membrane(X0, u)
    assert approx_equal(J, J0, margin) and np.allclose(f, J0 @ u, rtol=1e-12, atol=1e-6)


@pytest.mark.parametrize("sec", QP["transforms"], ids=lambda s: s["name"][:60])
def test_membrane_transformed_element(sec):
    a = sec["args"]
    if a[5] != 0.0 or a[6] != 0.0:
        pytest.skip("out-of-plane rotation: needs the local element frame "
                    "(geom_elem.cpp:358-374), outside the xy-plane membrane path")
    X = transform_element(X0, *a)
    f0, J0 = membrane(X0)
    f, J = membrane(X)
    margin = np.abs(J).mean() * QP["margin_factor"]
    Jfd = fd_jacobian(lambda u: membrane(X, u)[0], np.zeros(8), QP["fd_delta"])
    assert approx_equal(J, Jfd, margin)
    assert approx_equal(J, J.T)
    w = np.linalg.eigvalsh(J)
    assert np.sum(np.abs(w) < 1e-9 * np.abs(w).max()) == 3
    if "invariant to element" in sec["name"]:
        assert approx_equal(J, J0, margin)
    if "rotated about z" in sec["name"]:
        t = np.radians(a[7])
        R = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
        T = np.kron(R, np.eye(4))  # var-blocked rotation of (u, v)
        assert np.allclose(J, T @ J0 @ T.T, rtol=1e-10, atol=1e-6 * np.abs(J0).max())


# ----------------------------------------------------------------- HEX8
def test_hex8_rigid_modes_fd_and_symmetry():
    rng = np.random.default_rng(1)
    X, conn = O.grid_hex8(1, 1, 1)
    Xe = X[conn[0]] + rng.uniform(-0.1, 0.1, (8, 3))
    f, K = O.hex8_internal(Xe, 2.0, 0.3)
    w = np.linalg.eigvalsh(K)
    assert np.sum(np.abs(w) < 1e-10 * w.max()) == 6
    assert np.allclose(K, K.T, rtol=0, atol=1e-14 * np.abs(K).max())
    Jfd = fd_jacobian(lambda u: O.hex8_internal(Xe, 2.0, 0.3, u, want_K=False)[0], np.zeros(24),
                      QP["fd_delta"])
    assert approx_equal(K, Jfd, np.abs(Jfd).mean() * QP["margin_factor"])


def test_hex8_patch_test_reproduces_linear_field():
    """A linear displacement imposed on the boundary of a distorted patch is
    reproduced exactly at the interior node (the element passes the patch test)."""
    nx = ny = nz = 2
    X, conn = O.grid_hex8(nx, ny, nz)
    X = X.copy()
    center = 1 + 3 * (1 + 3 * 1)
    X[center] += np.array([0.13, -0.07, 0.11])
    rp, cols = O.csr_pattern(conn, X.shape[0], 3)
    fixed = np.ones(X.shape[0] * 3, dtype=np.uint8)
    fixed[center * 3:center * 3 + 3] = 0
    vals = O.assemble_hex8(X, conn, np.ones(conn.shape[0]), 0.3, rp, cols, None)
    A = sp.csr_matrix((vals, cols, rp)).toarray()
    G = np.array([[1e-3, 2e-3, -1e-3], [0.5e-3, -2e-3, 1e-3], [3e-3, 1e-3, 2e-3]])
    u_lin = (X @ G.T).reshape(-1)
    free = np.where(fixed == 0)[0]
    bnd = np.where(fixed == 1)[0]
    u_free = np.linalg.solve(A[np.ix_(free, free)], -A[np.ix_(free, bnd)] @ u_lin[bnd])
    assert np.allclose(u_free, u_lin[free], rtol=1e-10, atol=1e-14)


def test_simp_pcg_solution_matches_scipy_direct_solve():
    nx, ny, nz = 6, 3, 3
    rho = np.random.default_rng(2).uniform(0.05, 1.0, nx * ny * nz)
    d = O.simp_desc(nx, ny, nz, rtol=1e-13, maxit=100000)
    u, dc, rep = O.simp_solve(d, rho)
    X, conn = O.grid_hex8(nx, ny, nz)
    rp, cols = O.csr_pattern(conn, X.shape[0], 3)
    E, _ = O.simp_modulus(d, rho)
    fixed = O.simp_fixed_mask(d)
    vals = O.assemble_hex8(X, conn, E, 0.3, rp, cols, fixed)
    A = sp.csr_matrix((vals, cols, rp))
    F = O.simp_load_vector(d)
    u_ref = spla.spsolve(A.tocsc(), F)
    assert np.abs(u - u_ref).max() / np.abs(u_ref).max() < 1e-10
    assert abs(rep.compliance - F @ u_ref) / abs(F @ u_ref) < 1e-12


def test_compliance_sensitivity_matches_central_difference():
    """Design-gradient check in the manner of FunctionEvaluation::verify_gradients
    (src/optimization/function_evaluation.cpp:243+)."""
    nx, ny, nz = 6, 3, 3
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.2, 1.0, nx * ny * nz)
    d = O.simp_desc(nx, ny, nz, rtol=1e-14, maxit=100000)
    _, dc, _ = O.simp_solve(d, rho)
    for e in (0, 17, 40, 53):
        h = 1e-6
        r1 = rho.copy(); r1[e] += h
        r2 = rho.copy(); r2[e] -= h
        c1 = O.simp_solve(d, r1, False)[2].compliance
        c2 = O.simp_solve(d, r2, False)[2].compliance
        fd = (c1 - c2) / (2 * h)
        assert abs(fd - dc[e]) <= 1e-6 * abs(dc[e]) + 1e-12


# ----------------------------------------------------------------- heat
def test_heat_element_consistent_jacobian_matches_fd():
    rng = np.random.default_rng(4)
    X = np.array([[0, 0], [1.1, 0.1], [1.0, 0.9], [-0.1, 1.2]], float)
    T0 = rng.uniform(0, 5, 4)
    k0, beta, s, h = 1.3, 0.2, 0.9, 0.7

    def resid(T):
        return O.quad4_heat_internal(X, k0, beta, s, h, T, True, want_K=False)[0]
    _, K = O.quad4_heat_internal(X, k0, beta, s, h, T0, True)
    Jfd = fd_jacobian(resid, T0, 1e-3)
    assert np.allclose(K, Jfd, rtol=1e-9, atol=1e-12)
    fc, Kc = O.quad4_heat_convection(X, 1, 10.0, 0.5, h, T0)
    Jc = fd_jacobian(lambda T: O.quad4_heat_convection(X, 1, 10.0, 0.5, h, T)[0], T0, 1e-3)
    assert np.allclose(Kc, Jc, rtol=1e-10, atol=1e-12)


def test_heat_1d_analytic_solution():
    """Uniform source, constant k: -k T'' = q, T(0) = 0, -k T'(1) = h T(1).
    Bilinear elements reproduce the 1D solution at the nodes."""
    nx, ny = 20, 4
    d = O.heat_desc(nx=nx, ny=ny, beta=0.0, rtol=1e-13)
    T, _, _ = O.heat_solve(d, None, np.ones(nx * ny), want_sens=False)
    x = np.linspace(0, 1, nx + 1)
    exact = -x ** 2 / 2 + 6 * x / 11
    assert np.allclose(T.reshape(ny + 1, nx + 1), exact[None, :], rtol=0, atol=1e-12)


def test_heat_adjoint_sensitivities_match_fd():
    nx = ny = 10
    q = O.heat_source_field(nx, ny)
    d = O.heat_desc(nx=nx, ny=ny, rtol=1e-14, newton_rtol=1e-14)
    s = np.random.default_rng(5).uniform(0.5, 1.5, nx * ny)
    _, ds, rep = O.heat_solve(d, s, q)
    for e in (0, 37, 55):
        h = 1e-6
        s1 = s.copy(); s1[e] += h
        s2 = s.copy(); s2[e] -= h
        fd = (O.heat_solve(d, s1, q, False)[2].mean_temperature -
              O.heat_solve(d, s2, q, False)[2].mean_temperature) / (2 * h)
        assert abs(fd - ds[e]) <= 1e-5 * abs(ds[e]) + 5e-11  # FD noise of q ~ 1e-17 / h
    h = 1e-6
    d1 = O.heat_desc(nx=nx, ny=ny, k0=1 + h, rtol=1e-14, newton_rtol=1e-14)
    d2 = O.heat_desc(nx=nx, ny=ny, k0=1 - h, rtol=1e-14, newton_rtol=1e-14)
    fd = (O.heat_solve(d1, s, q, False)[2].mean_temperature -
          O.heat_solve(d2, s, q, False)[2].mean_temperature) / (2 * h)
    assert abs(fd - rep.dq_dk0) <= 1e-6 * abs(rep.dq_dk0)
