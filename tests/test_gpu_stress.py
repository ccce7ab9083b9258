"""KS-aggregated von Mises stress output (mg_ks_stress) against the FP64 oracle.

The GPU output is evaluated at the oracle's own solution, so the comparison covers the
stress kernels, the reductions and the adjoint, not the primal solve.  Tolerances: the
KS value and the largest von Mises stress to 1e-12 relative; the total density
derivative (adjoint CG to 1e-13) to 1e-9 relative.
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def cantilever_arrays(nx, ny, nz, load):
    """mesh, Dirichlet mask and load vector of mastgpu.simp_cantilever"""
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


def simp(rho, penal, E0=1.0, Emin=1e-9):
    rmin = Emin / E0
    return E0 * (rmin + (1 - rmin) * rho ** penal), E0 * (1 - rmin) * penal * rho ** (penal - 1)


def test_ks_stress_linear_matches_oracle():
    nx, ny, nz = 6, 3, 3
    rho = np.random.default_rng(11).uniform(0.3, 1.0, nx * ny * nz)
    coords, conn, fixed, F = cantilever_arrays(nx, ny, nz, 1.0)
    E, dE = simp(rho, 3.0)
    Es, dEs = simp(rho, 0.5)
    rp, cl = O.csr_pattern(conn, coords.shape[0], 3)
    u, _, _ = O.pcg(rp, cl, O.assemble_hex8(coords, conn, E, 0.3, rp, cl, fixed), F, 1e-15, 100000)
    p_ks, s0 = 8.0, 1.0
    q_ref, vmax_ref, d_ref = O.ks_stress_total_sensitivity(coords, conn, E, dE, Es, dEs, 0.3, u, fixed,
                                                           p_ks, s0)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        q, vmax, d = p.ks_stress(p_ks, s0, stress_penalty=0.5, X=u)
        q2, vmax2, _ = p.ks_stress(p_ks, s0, stress_penalty=0.5, X=u, want_sens=False)
    assert abs(q - q_ref) <= 1e-12 * max(abs(q_ref), 1.0)
    assert abs(vmax - vmax_ref) <= 1e-12 * vmax_ref
    assert rel(d, d_ref) < 1e-9
    assert q2 == q and vmax2 == vmax  # deterministic reductions


def test_ks_stress_after_a_solve_uses_the_resident_solution():
    nx, ny, nz = 6, 3, 3
    rho = np.full(nx * ny * nz, 0.8)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        u, _ = p.solve(M.default_opts(rtol=1e-12))
        q_res, vmax_res, d_res = p.ks_stress(8.0, 1.0, stress_penalty=0.5)
        q_x, vmax_x, d_x = p.ks_stress(8.0, 1.0, stress_penalty=0.5, X=u)
    assert q_res == q_x and vmax_res == vmax_x
    assert rel(d_res, d_x) < 1e-12


def test_ks_stress_nonlinear_strain_matches_oracle():
    nx, ny, nz, load = 6, 2, 2, 0.01
    rho = np.linspace(0.7, 1.0, nx * ny * nz)
    coords, conn, fixed, F = cantilever_arrays(nx, ny, nz, load)
    E, dE = simp(rho, 3.0)
    Es, dEs = simp(rho, 0.5)
    u, _ = O.newton_hex8_gl(coords, conn, E, 0.3, F, fixed, rtol=1e-13)
    p_ks, s0 = 6.0, 0.01
    q_ref, vmax_ref, d_ref = O.ks_stress_total_sensitivity(coords, conn, E, dE, Es, dEs, 0.3, u, fixed,
                                                           p_ks, s0, nonlinear=True)
    with M.simp_cantilever(nx, ny, nz, physics=M.PHYS_HEX8_NONLINEAR, load=load) as p:
        p.set_design(rho)
        q, vmax, d = p.ks_stress(p_ks, s0, stress_penalty=0.5, X=u)
    assert abs(q - q_ref) <= 1e-12 * max(abs(q_ref), 1.0)
    assert abs(vmax - vmax_ref) <= 1e-12 * vmax_ref
    assert rel(d, d_ref) < 1e-9


def test_ks_stress_rejects_bad_arguments_and_other_physics():
    with M.simp_cantilever(2, 1, 1) as p:
        for bad in ((0.0, 1.0), (8.0, 0.0), (-1.0, 1.0)):
            with pytest.raises(M.MastGpuError) as err:
                p.ks_stress(*bad)
            assert err.value.status == M.MG_EINVAL
    coords, conn = M.grid_quad4(2, 2)
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, M.SIMP_MATERIAL) as p:
        with pytest.raises(M.MastGpuError) as err:
            p.ks_stress(8.0, 1.0)
        assert err.value.status == M.MG_ENOTSUP
