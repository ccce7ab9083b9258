"""Geometrically nonlinear HEX8 (Green-Lagrange strain, MAST::NONLINEAR_STRAIN) through
the C ABI against the FP64 oracle.

Tolerances as for the plain linear form: element matrices, internal forces and the
global residual to 1e-12 relative; Newton solution, compliance and sensitivities to
1e-10 relative.
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu

RTOL_ELEM = 1e-12
RTOL_SOL = 1e-10
NL = M.PHYS_HEX8_NONLINEAR


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def cantilever_arrays(nx, ny, nz, load):
    """The mesh, Dirichlet mask and load vector of mastgpu.simp_cantilever."""
    coords, conn = O.grid_hex8(nx, ny, nz)
    NX, NY = nx + 1, ny + 1
    fixed = np.zeros(coords.shape[0] * 3, np.uint8)
    F = np.zeros(coords.shape[0] * 3)
    for k in range(nz + 1):
        for j in range(NY):
            fixed[(NX * (j + NY * k)) * 3 + np.arange(3)] = 1
    for j in range(ny + 1):
        F[(nx + NX * j) * 3 + 2] += -load / (ny + 1)
    return coords, conn, fixed, F


@pytest.mark.parametrize("scale", [0.0, 0.08])
def test_element_tangent_and_force(scale):
    rng = np.random.default_rng(5)
    coords, conn = M.grid_hex8(2, 1, 1)
    coords = coords + rng.uniform(-0.12, 0.12, coords.shape)
    rho = rng.uniform(0.2, 1.0, conn.shape[0])
    X = rng.normal(scale=scale, size=coords.shape[0] * 3)
    with M.Problem(NL, coords, conn, M.SIMP_MATERIAL) as p:
        p.set_design(rho)
        Ke, fe = p.element_matrices(0, conn.shape[0], X)
    E, _ = O.simp_modulus(O.simp_desc(1, 1, 1), rho)
    for e in range(conn.shape[0]):
        ue = X.reshape(-1, 3)[conn[e]].T.reshape(-1)
        f_ref, K_ref = O.hex8_internal_gl(coords[conn[e]], E[e], 0.3, ue)
        assert rel(Ke[e], K_ref) < RTOL_ELEM
        if scale > 0:
            assert rel(fe[e], f_ref) < RTOL_ELEM
        else:
            assert np.abs(fe[e]).max() == 0.0


def test_csr_tangent_and_residual_match_oracle():
    nx, ny, nz = 5, 3, 2
    rng = np.random.default_rng(6)
    rho = rng.uniform(0.05, 1.0, nx * ny * nz)
    coords, conn, fixed, F = cantilever_arrays(nx, ny, nz, 1.0)
    X = rng.normal(scale=0.05, size=coords.shape[0] * 3)
    X[fixed == 1] = 0.0
    with M.simp_cantilever(nx, ny, nz, physics=NL) as p:
        p.set_design(rho)
        R = p.residual_and_jacobian(X)
        rowptr, cols, vals = p.get_csr()
    rp_ref, cols_ref = O.csr_pattern(conn, coords.shape[0], 3)
    assert np.array_equal(rowptr, rp_ref) and np.array_equal(cols, cols_ref)
    E, _ = O.simp_modulus(O.simp_desc(nx, ny, nz), rho)
    vals_ref, R_ref = O.assemble_hex8_gl(coords, conn, E, 0.3, X, F, rp_ref, cols_ref, fixed)
    assert rel(vals, vals_ref) < RTOL_ELEM
    assert rel(R, R_ref) < RTOL_ELEM


def test_newton_large_deflection_matches_oracle():
    nx, ny, nz, load = 8, 2, 2, 0.02
    rho = np.linspace(0.6, 1.0, nx * ny * nz)
    coords, conn, fixed, F = cantilever_arrays(nx, ny, nz, load)
    E, dE = O.simp_modulus(O.simp_desc(nx, ny, nz), rho)
    u_ref, hist = O.newton_hex8_gl(coords, conn, E, 0.3, F, fixed, rtol=1e-12)
    with M.simp_cantilever(nx, ny, nz, physics=NL, load=load) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(newton_rtol=1e-12, rtol=1e-12))
        assert rep.newton_iterations >= 3  # a nonlinear solve, not one linear step
        assert abs(rep.newton_iterations - (len(hist) - 1)) <= 1
        c, dc = p.compliance()
    assert rel(u, u_ref) < RTOL_SOL
    assert abs(c - F @ u_ref) <= RTOL_SOL * abs(F @ u_ref)
    dc_ref = O.hex8_gl_compliance_sens(coords, conn, dE, 0.3, u_ref, E, F, fixed)
    assert rel(dc, dc_ref) < RTOL_SOL


def test_small_load_reduces_to_the_linear_solve():
    nx, ny, nz, load = 6, 2, 2, 1e-7
    with M.simp_cantilever(nx, ny, nz, physics=NL, load=load) as p:
        u_nl, _ = p.solve(M.default_opts(newton_rtol=1e-12, rtol=1e-12))
    with M.simp_cantilever(nx, ny, nz, load=load) as p:
        u_lin, _ = p.solve(M.default_opts(rtol=1e-12))
    assert rel(u_nl, u_lin) < 1e-5


def test_density_residual_sensitivity():
    """dR/drho_e = dE_e f1_e(X) scattered (free rows), through mg_sensitivity_assemble."""
    nx, ny, nz = 3, 2, 2
    rng = np.random.default_rng(7)
    rho = rng.uniform(0.2, 1.0, nx * ny * nz)
    coords, conn, fixed, _ = cantilever_arrays(nx, ny, nz, 1.0)
    X = rng.normal(scale=0.05, size=coords.shape[0] * 3)
    X[fixed == 1] = 0.0
    _, dE = O.simp_modulus(O.simp_desc(nx, ny, nz), rho)
    with M.simp_cantilever(nx, ny, nz, physics=NL) as p:
        p.set_design(rho)
        for e in (0, 5, nx * ny * nz - 1):
            g = p.sensitivity_assemble(M.PARAM_DENSITY, e, X)
            ref = np.zeros_like(g)
            ue = X.reshape(-1, 3)[conn[e]].T.reshape(-1)
            f1, _ = O.hex8_internal_gl(coords[conn[e]], 1.0, 0.3, ue, want_K=False)
            for a in range(8):
                for i in range(3):
                    ref[conn[e][a] * 3 + i] += dE[e] * f1[i * 8 + a]
            ref[fixed == 1] = 0.0
            assert rel(g, ref) < RTOL_ELEM


def test_mixed_precision_is_refused_for_the_nonlinear_form():
    with M.simp_cantilever(4, 2, 2, physics=NL) as p:
        with pytest.raises(M.MastGpuError) as err:
            p.solve(M.default_opts(precision=M.MIXED_TF32X3))
        assert err.value.status == M.MG_ENOTSUP
