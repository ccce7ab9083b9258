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


# ---------------------------------------------------------------- device source on the host
def _host_element():
    import ctypes
    import os
    import subprocess
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = os.path.join(repo, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libgl_element_host.so")
    src = os.path.join(repo, "tests", "cpp", "gl_element_host.cpp")
    hdr = os.path.join(repo, "mast-multiphysics_gb300", "csrc", "hex8_gl.cuh")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                            "-x", "c++", "-I", os.path.dirname(hdr), src, "-o", so],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.gl_element_host.argtypes = [p, ctypes.c_double, ctypes.c_double, p, p, p]
    return L


@pytest.mark.parametrize("distort,scale", [(0.0, 0.0), (0.1, 0.05), (0.15, 0.3)])
def test_device_element_source_matches_the_oracle(distort, scale):
    """The phases of the CUDA element (hex8_gl.cuh), run lane by lane on the host,
    against the oracle's 6 x 24 strain-operator form: FP64 round-off only."""
    L = _host_element()
    X = element(distort, seed=3)
    u = np.random.default_rng(4).normal(scale=scale, size=24)
    f = np.zeros(24)
    K = np.zeros(576)
    assert L.gl_element_host(np.ascontiguousarray(X.reshape(24)), 3.0, 0.3, u, f, K) == 0
    fo, Ko = O.hex8_internal_gl(X, 3.0, 0.3, u)
    K = K.reshape(24, 24)
    assert np.abs(K - Ko).max() <= 1e-12 * np.abs(Ko).max()
    assert np.abs(f - fo).max() <= 1e-12 * max(np.abs(fo).max(), np.abs(Ko).max() * max(scale, 1e-3))


@pytest.mark.parametrize("scale", [1e-6, 1e-9])
def test_device_element_source_keeps_small_strains(scale):
    """Tiny displacements: the internal force must keep its relative accuracy (a strain
    formed as (Fd^T Fd - I)/2 would lose the digits that cancel against the identity)."""
    L = _host_element()
    X = element(0.1, seed=5)
    u = np.random.default_rng(6).normal(scale=scale, size=24)
    f = np.zeros(24)
    K = np.zeros(576)
    assert L.gl_element_host(np.ascontiguousarray(X.reshape(24)), 1.0, 0.3, u, f, K) == 0
    fo, _ = O.hex8_internal_gl(X, 1.0, 0.3, u)
    assert np.abs(f - fo).max() <= 1e-12 * np.abs(fo).max()


# ---------------------------------------------------------------- global system
def beam(nx=4, ny=1, nz=1, load=0.02):
    coords, conn = O.grid_hex8(nx, ny, nz)
    nn = coords.shape[0]
    fixed = np.zeros(nn * 3, np.uint8)
    F = np.zeros(nn * 3)
    tip = np.where(coords[:, 0] == nx)[0]
    fixed[(np.where(coords[:, 0] == 0)[0][:, None] * 3 + np.arange(3)).reshape(-1)] = 1
    F[tip * 3 + 2] = -load / tip.shape[0]
    return coords, conn, fixed, F


def test_newton_small_load_gives_the_linear_solution():
    coords, conn, fixed, F = beam(load=1e-7)
    E = np.full(conn.shape[0], 1.0)
    u, hist = O.newton_hex8_gl(coords, conn, E, 0.3, F, fixed)
    rowptr, cols = O.csr_pattern(conn, coords.shape[0], 3)
    vals = O.assemble_hex8(coords, conn, E, 0.3, rowptr, cols, fixed)
    ul, _, _ = O.pcg(rowptr, cols, vals, F, 1e-14, 10000)
    assert np.abs(u - ul).max() <= 1e-5 * np.abs(ul).max()


def test_newton_converges_quadratically_under_a_large_load():
    coords, conn, fixed, F = beam(load=0.05)
    u, hist = O.newton_hex8_gl(coords, conn, np.full(conn.shape[0], 1.0), 0.3, F, fixed)
    assert hist[-1] <= 1e-10 * hist[0]
    # the last steps square the residual (up to the Krylov tolerance)
    r = np.array(hist) / hist[0]
    k = int(np.argmax(r < 1e-3))
    assert r[k + 1] <= 10 * r[k] ** 1.8 or r[k + 1] <= 1e-10
    # rotation of the tip: the deflection differs from the linear one
    rowptr, cols = O.csr_pattern(conn, coords.shape[0], 3)
    vals = O.assemble_hex8(coords, conn, np.full(conn.shape[0], 1.0), 0.3, rowptr, cols, fixed)
    ul, _, _ = O.pcg(rowptr, cols, vals, F, 1e-14, 10000)
    assert abs(np.abs(u).max() - np.abs(ul).max()) > 0.02 * np.abs(ul).max()


def test_adjoint_compliance_sensitivity_matches_finite_differences():
    coords, conn, fixed, F = beam(nx=3, load=0.03)
    d = O.simp_desc(3, 1, 1)
    rho = np.array([0.9, 0.6, 0.75])

    def compliance(r):
        E, _ = O.simp_modulus(d, r)
        u, _ = O.newton_hex8_gl(coords, conn, E, 0.3, F, fixed, rtol=1e-14)
        return float(F @ u), u

    c0, u0 = compliance(rho)
    E, dE = O.simp_modulus(d, rho)
    dc = O.hex8_gl_compliance_sens(coords, conn, dE, 0.3, u0, E, F, fixed)
    h = 1e-5
    for e in range(3):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (compliance(rp)[0] - compliance(rm)[0]) / (2 * h)
        assert abs(dc[e] - fd) <= 1e-6 * abs(fd)


def test_internal_force_is_the_strain_energy_gradient():
    """St Venant-Kirchhoff is hyperelastic: f_int = dPi/du with Pi = sum_qp JxW E:C:E / 2 over
    the Green-Lagrange strain (computed here independently, by numpy from the shape data)."""
    X = element(0.1, seed=9)
    u = np.random.default_rng(10).normal(scale=0.08, size=24)
    E, nu = 3.0, 0.25
    C = O.iso_stiffness_3d(E, nu)
    g = 1 / np.sqrt(3)
    signs = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                      [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)

    def energy(uv):
        disp = uv.reshape(3, 8).T
        Pi = 0.0
        for q in range(8):
            xi = np.array([q & 1, q >> 1 & 1, q >> 2 & 1]) * 2 * g - g
            dN = np.array([[s[d] / 8 * np.prod([1 + s[k] * xi[k] for k in range(3) if k != d])
                            for d in range(3)] for s in signs])  # (8, 3) reference gradients
            J = dN.T @ X
            gN = dN @ np.linalg.inv(J).T
            H = disp.T @ gN
            Eg = 0.5 * (H + H.T + H.T @ H)
            ev = np.array([Eg[0, 0], Eg[1, 1], Eg[2, 2], 2 * Eg[0, 1], 2 * Eg[1, 2], 2 * Eg[0, 2]])
            Pi += np.linalg.det(J) * 0.5 * ev @ C @ ev
        return Pi

    f, _ = O.hex8_internal_gl(X, E, nu, u, want_K=False)
    h = 1e-6
    grad = np.array([(energy(u + h * np.eye(24)[c]) - energy(u - h * np.eye(24)[c])) / (2 * h)
                     for c in range(24)])
    assert np.abs(f - grad).max() <= 1e-7 * np.abs(f).max()
