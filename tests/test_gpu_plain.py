"""Plain FP64 form: CUDA kernels through the C ABI vs the FP64 oracle.

Tolerances (stated by the spec of this path): element matrices and the global
residual to 1e-12 relative; solution, compliance and sensitivities to 1e-10
relative.
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu

RTOL_ELEM = 1e-12
RTOL_SOL = 1e-10


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def distorted_hex8(seed=3):
    rng = np.random.default_rng(seed)
    coords, conn = M.grid_hex8(2, 1, 1)
    coords = coords + rng.uniform(-0.15, 0.15, coords.shape)
    return coords, conn


@pytest.mark.parametrize("distort", [False, True])
def test_hex8_element_matrices(distort):
    coords, conn = distorted_hex8() if distort else M.grid_hex8(2, 1, 1)
    rng = np.random.default_rng(1)
    rho = rng.uniform(0.1, 1.0, conn.shape[0])
    X = rng.standard_normal(coords.shape[0] * 3)
    with M.Problem(M.PHYS_HEX8, coords, conn, M.SIMP_MATERIAL) as p:
        p.set_design(rho)
        Ke, fe = p.element_matrices(0, conn.shape[0], X)
    d = O.simp_desc(1, 1, 1)
    E, _ = O.simp_modulus(d, rho)
    for e in range(conn.shape[0]):
        Xe = coords[conn[e]]
        ue = X.reshape(-1, 3)[conn[e]].T.reshape(-1)  # var-blocked
        f_ref, K_ref = O.hex8_internal(Xe, E[e], 0.3, ue)
        assert rel(Ke[e], K_ref) < RTOL_ELEM
        assert rel(fe[e], f_ref) < RTOL_ELEM


def test_hex8_csr_and_residual_match_oracle():
    nx, ny, nz = 5, 3, 2
    rng = np.random.default_rng(2)
    rho = rng.uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        X = rng.standard_normal(p.n_dofs)
        fixed = O.simp_fixed_mask(O.simp_desc(nx, ny, nz))
        X[fixed == 1] = 0.0
        R = p.residual_and_jacobian(X)
        rowptr, cols, vals = p.get_csr()
    coords, conn = O.grid_hex8(nx, ny, nz)
    rp_ref, cols_ref = O.csr_pattern(conn, coords.shape[0], 3)
    assert np.array_equal(rowptr, rp_ref) and np.array_equal(cols, cols_ref)
    d = O.simp_desc(nx, ny, nz)
    E, _ = O.simp_modulus(d, rho)
    vals_ref = O.assemble_hex8(coords, conn, E, 0.3, rp_ref, cols_ref, fixed)
    assert rel(vals, vals_ref) < RTOL_ELEM
    F = O.simp_load_vector(d)
    R_ref = O.spmv(rp_ref, cols_ref, vals_ref, X) - F
    R_ref[fixed == 1] = X[fixed == 1]
    assert rel(R, R_ref) < RTOL_ELEM


def test_cantilever_24x12x12_matches_oracle():
    """The CPU-runnable plain-method workload: 24x12x12, rho = 0.5, rtol 1e-10."""
    nx, ny, nz = 24, 12, 12
    rho = np.full(nx * ny * nz, 0.5)
    with M.simp_cantilever(nx, ny, nz) as p:
        assert p.n_dofs == 12675 and p.nnz == 899433
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-12))
        c, dc = p.compliance()
    assert rep.status == 0 and rep.relres <= 1e-12
    u_ref, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-13), rho)
    assert rel(u, u_ref) < RTOL_SOL
    assert abs(c - r.compliance) / abs(r.compliance) < RTOL_SOL
    assert rel(dc, dc_ref) < RTOL_SOL


def test_cantilever_rtol_1e10_iterations_and_relres():
    nx, ny, nz = 24, 12, 12
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(np.full(nx * ny * nz, 0.5))
        u, rep = p.solve(M.default_opts(rtol=1e-10))
    _, _, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-10), np.full(nx * ny * nz, 0.5), False)
    assert rep.relres <= 1.0001e-10
    # same algorithm (Jacobi-PCG, same stopping rule): iteration counts agree closely
    assert abs(rep.krylov_iterations - r.iterations) <= 2


def test_random_density_sensitivity_vs_oracle():
    nx, ny, nz = 8, 4, 4
    rho = np.random.default_rng(11).uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-13, max_iterations=100000))
        c, dc = p.compliance()
    u_ref, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-14, maxit=400000), rho)
    assert rel(u, u_ref) < RTOL_SOL
    assert abs(c - r.compliance) / r.compliance < RTOL_SOL
    assert rel(dc, dc_ref) < RTOL_SOL


def test_assembly_is_deterministic():
    nx, ny, nz = 6, 4, 4
    rho = np.random.default_rng(5).uniform(0.01, 1.0, nx * ny * nz)
    out = []
    for _ in range(2):
        with M.simp_cantilever(nx, ny, nz) as p:
            p.set_design(rho)
            u, _ = p.solve(M.default_opts(rtol=1e-10))
            out.append((p.get_csr()[2].copy(), u))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_heat_element_matrices():
    coords, conn = M.grid_quad4(3, 2)
    rng = np.random.default_rng(4)
    coords = coords + rng.uniform(-0.05, 0.05, coords.shape)
    T = rng.uniform(0, 2.0, coords.shape[0])
    src = rng.uniform(0, 1, conn.shape[0])
    mat = dict(E0=0.0, Emin=0.0, nu=0.0, penal=1.0, thickness=0.7, k0=1.3, k_beta=0.05)
    with M.Problem(M.PHYS_HEAT, coords, conn, mat, source_elem=src) as p:
        s = rng.uniform(0.5, 1.5, conn.shape[0])
        p.set_elem_scale(s)
        Ke, fe = p.element_matrices(0, conn.shape[0], T)
    for e in range(conn.shape[0]):
        Xe = coords[conn[e]]
        f_ref, K_ref = O.quad4_heat_internal(Xe, 1.3, 0.05, s[e], 0.7, T[conn[e]], True)
        f_ref = f_ref + O.quad4_heat_source(Xe, src[e], 0.7)
        assert rel(Ke[e], K_ref) < RTOL_ELEM
        assert rel(fe[e], f_ref) < RTOL_ELEM


def test_heat_newton_and_adjoint_match_oracle():
    """Nonlinear conduction on QUAD4 200x200 (k = k0 (1 + 0.01 T), q = 1 on
    [0.25,0.75]^2, T = 0 at x = 0, h = 10 convection at x = 1)."""
    with M.heat_square(200, 200) as p:
        assert p.n_dofs == 40401 and p.nnz == 361201
        T, rep = p.solve(M.default_opts(rtol=1e-12, newton_rtol=1e-11, krylov=M.KRYLOV_CG))
        q, dk0, ds = p.mean_temperature(opts=M.default_opts(rtol=1e-12, krylov=M.KRYLOV_BICGSTAB))
    T_ref, ds_ref, hr = O.heat_solve(O.heat_desc(rtol=1e-12, newton_rtol=1e-11, krylov=0),
                                     None, O.heat_source_field(200, 200))
    assert rep.status == 0
    assert rel(T, T_ref) < RTOL_SOL
    assert abs(q - hr.mean_temperature) / abs(hr.mean_temperature) < RTOL_SOL
    assert abs(dk0 - hr.dq_dk0) / abs(hr.dq_dk0) < RTOL_SOL
    assert rel(ds, ds_ref) < RTOL_SOL


def test_membrane_element_matrices():
    coords = np.array([[-1.0, -1.0], [1.0, -1.0], [1.0, 1.0], [-1.0, 1.0]])
    conn = np.array([[0, 1, 2, 3]], dtype=np.int32)
    mat = dict(E0=72e9, Emin=0.0, nu=0.33, penal=1.0, thickness=0.06, k0=0.0, k_beta=0.0)
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, mat) as p:
        Ke, _ = p.element_matrices(0, 1)
    _, K_ref = O.quad4_membrane_internal(coords, 72e9, 0.33, 0.06)
    assert rel(Ke[0], K_ref) < RTOL_ELEM


def test_bad_inputs_return_status():
    nx, ny, nz = 3, 2, 2
    with M.simp_cantilever(nx, ny, nz) as p:
        rho = np.full(nx * ny * nz, 0.5)
        rho[3] = np.nan
        with pytest.raises(M.MastGpuError) as ei:
            p.set_design(rho)
        assert ei.value.status == M.MG_EINVAL
    coords, conn = M.grid_hex8(2, 1, 1)
    bad = conn.copy()
    bad[1, 3] = 10 ** 6
    with pytest.raises(M.MastGpuError) as ei:
        M.Problem(M.PHYS_HEX8, coords, bad, M.SIMP_MATERIAL)
    assert ei.value.status == M.MG_EINVAL


def test_injected_allocation_failure_is_reported():
    L = M.lib()
    L.mg_debug_fail_alloc_after(3)
    try:
        with pytest.raises(M.MastGpuError) as ei:
            M.simp_cantilever(4, 2, 2)
        assert ei.value.status == M.MG_ENOMEM
    finally:
        L.mg_debug_fail_alloc_after(-1)
    with M.simp_cantilever(4, 2, 2) as p:  # library still usable
        p.solve()


def test_iteration_cap_reports_enoconv():
    with M.simp_cantilever(8, 4, 4) as p:
        _, rep = p.solve(M.default_opts(rtol=1e-12, max_iterations=5), raise_on_error=False)
    assert rep.status == M.MG_ENOCONV
