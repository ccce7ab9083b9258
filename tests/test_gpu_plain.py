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


def test_nodal_density_field_vs_oracle():
    """MAST example 6's design is a nodal (FIRST-order LAGRANGE) density read
    through MeshFieldFunction: the modulus at each Gauss point from the trilinear
    field.  Solution, compliance and dC/drho per node against the oracle's nodal
    path; element matrices against the oracle element with per-point moduli; the
    mixed-precision solve refuses a nodal field."""
    nx, ny, nz = 8, 4, 4
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    rho = np.random.default_rng(12).uniform(0.05, 1.0, nn)
    desc = O.simp_desc(nx, ny, nz, rtol=1e-14, maxit=400000)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design_nodal(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-13, max_iterations=100000))
        c, dc = p.compliance()
        Ke = p.element_matrices(5, 1)[0][0]
        with pytest.raises(M.MastGpuError):
            p.solve(M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8))
        conn = p.conn.copy()
        coords = p.coords.copy()
    u_ref, dc_ref, r = O.simp_solve_nodal(desc, rho)
    assert dc.shape == (nn,)
    assert rel(u, u_ref) < RTOL_SOL
    assert abs(c - r.compliance) / r.compliance < RTOL_SOL
    assert rel(dc, dc_ref) < RTOL_SOL
    Eq, _ = O.simp_nodal_modulus(desc, conn[5:6], rho)
    X = coords[conn[5]].ravel()
    _, K_ref = O.hex8_internal_qp(X, Eq[0], 0.3, np.zeros(24))
    assert np.abs(Ke - K_ref).max() <= 1e-12 * np.abs(K_ref).max()


def test_design_outside_the_unit_interval_is_rejected():
    """mg_set_design: the modulus kernel flags densities outside [0,1] or NaN;
    the call returns MG_EINVAL naming the first such element."""
    with M.simp_cantilever(4, 2, 2) as p:
        rho = np.full(16, 0.5)
        rho[9] = 1.5
        with pytest.raises(M.MastGpuError) as ei:
            p.set_design(rho)
        assert ei.value.status == M.MG_EINVAL and "density 9" in str(ei.value)
        rho[9] = np.nan
        with pytest.raises(M.MastGpuError):
            p.set_design(rho)
        p.set_design(np.full(16, 0.5))  # and a valid design is taken afterwards
        u, rep = p.solve(M.default_opts(rtol=1e-10))
        assert rep.status == 0


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


MEMBRANE_MAT = dict(E0=72e9, Emin=72e9 * 1e-9, nu=0.33, penal=3.0, thickness=0.06, k0=0.0,
                    k_beta=0.0)


def distorted_quad4(nx, ny, lx, ly, seed):
    """A QUAD4 grid with every interior node moved by up to 20 % of a cell."""
    coords, conn = M.grid_quad4(nx, ny, lx, ly)
    rng = np.random.default_rng(seed)
    hx, hy = lx / nx, ly / ny
    i = np.arange(coords.shape[0]) % (nx + 1)
    j = np.arange(coords.shape[0]) // (nx + 1)
    inner = (i > 0) & (i < nx) & (j > 0) & (j < ny)
    coords[inner, 0] += rng.uniform(-0.2, 0.2, inner.sum()) * hx
    coords[inner, 1] += rng.uniform(-0.2, 0.2, inner.sum()) * hy
    return coords, conn


def membrane_modulus(rho):
    m = MEMBRANE_MAT
    rmin = m["Emin"] / m["E0"]
    return m["E0"] * (rmin + (1.0 - rmin) * rho ** m["penal"])


def test_membrane_distorted_elements_at_a_displacement():
    """Distorted QUAD4 membranes with per-element moduli, K_e and f_e = K_e u_e at a
    random displacement (StructuralElement2D::internal_residual, membrane part)."""
    coords, conn = distorted_quad4(4, 3, 2.0, 1.0, seed=5)
    rng = np.random.default_rng(6)
    rho = rng.uniform(0.1, 1.0, conn.shape[0])
    X = rng.standard_normal(coords.shape[0] * 2) * 1e-3
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, MEMBRANE_MAT) as p:
        p.set_design(rho)
        Ke, fe = p.element_matrices(0, conn.shape[0], X)
    E = membrane_modulus(rho)
    for e in range(conn.shape[0]):
        ue = np.concatenate([X[conn[e] * 2], X[conn[e] * 2 + 1]])  # var-blocked (u | v)
        f_ref, K_ref = O.quad4_membrane_internal(coords[conn[e]], E[e], 0.33, 0.06, ue)
        assert rel(Ke[e], K_ref) < RTOL_ELEM
        assert rel(fe[e], f_ref) < RTOL_ELEM


def membrane_cantilever(nx, ny, seed):
    """Plane-stress cantilever: x = 0 edge clamped, a unit -y load spread over the
    x = lx edge; distorted interior nodes, random densities."""
    lx, ly = 4.0, 1.0
    coords, conn = distorted_quad4(nx, ny, lx, ly, seed)
    nodes = np.arange(coords.shape[0])
    left = nodes[nodes % (nx + 1) == 0]
    right = nodes[nodes % (nx + 1) == nx]
    fixed_dofs = np.sort(np.concatenate([2 * left, 2 * left + 1]))
    load_dofs = 2 * right + 1
    load_values = np.full(right.shape[0], -1.0 / right.shape[0])
    rho = np.random.default_rng(seed + 1).uniform(0.05, 1.0, conn.shape[0])
    return coords, conn, fixed_dofs, load_dofs, load_values, rho


def test_membrane_csr_and_residual_match_oracle():
    coords, conn, fixed_dofs, load_dofs, load_values, rho = membrane_cantilever(9, 4, seed=8)
    n = coords.shape[0] * 2
    rng = np.random.default_rng(9)
    X = rng.standard_normal(n)
    X[fixed_dofs] = 0.0
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, MEMBRANE_MAT, fixed_dofs=fixed_dofs,
                   load_dofs=load_dofs, load_values=load_values) as p:
        p.set_design(rho)
        R = p.residual_and_jacobian(X)
        rowptr, cols, vals = p.get_csr()
    rp_ref, cols_ref = O.csr_pattern(conn, coords.shape[0], 2)
    assert np.array_equal(rowptr, rp_ref) and np.array_equal(cols, cols_ref)
    fixed = np.zeros(n, dtype=np.uint8)
    fixed[fixed_dofs] = 1
    vals_ref = O.assemble_quad4_membrane(coords, conn, membrane_modulus(rho), 0.33, 0.06,
                                         rp_ref, cols_ref, fixed)
    assert rel(vals, vals_ref) < RTOL_ELEM
    F = np.zeros(n)
    F[load_dofs] = load_values
    R_ref = O.spmv(rp_ref, cols_ref, vals_ref, X) - F
    R_ref[fixed_dofs] = X[fixed_dofs]
    assert rel(R, R_ref) < RTOL_ELEM


def test_membrane_cantilever_solve_matches_oracle():
    """Assembled QUAD4 membrane solve (plain FP64 CG) against the oracle's own
    assembly and Jacobi-PCG: solution and compliance to 1e-10."""
    coords, conn, fixed_dofs, load_dofs, load_values, rho = membrane_cantilever(40, 10, seed=11)
    n = coords.shape[0] * 2
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, MEMBRANE_MAT, fixed_dofs=fixed_dofs,
                   load_dofs=load_dofs, load_values=load_values) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-13, krylov=M.KRYLOV_CG, max_iterations=200000))
    assert rep.status == 0
    fixed = np.zeros(n, dtype=np.uint8)
    fixed[fixed_dofs] = 1
    rp, cols = O.csr_pattern(conn, coords.shape[0], 2)
    vals = O.assemble_quad4_membrane(coords, conn, membrane_modulus(rho), 0.33, 0.06, rp, cols,
                                     fixed)
    F = np.zeros(n)
    F[load_dofs] = load_values
    u_ref, it, rr = O.pcg(rp, cols, vals, F, 1e-14, 10 ** 6)
    assert rr < 1e-13
    assert rel(u, u_ref) < RTOL_SOL
    assert abs(F @ u - F @ u_ref) / abs(F @ u_ref) < RTOL_SOL


def test_sensitivity_solve_matches_fd_and_the_adjoint():
    """J du/drho_e = -dR/drho_e (NonlinearSystem::sensitivity_solve): the direct compliance
    sensitivity F . du/drho_e equals the adjoint dC/drho_e, and du/drho_e matches central
    differences of re-solved displacements."""
    nx, ny, nz = 6, 3, 3
    rho = np.random.default_rng(21).uniform(0.1, 1.0, nx * ny * nz)
    opts = M.default_opts(rtol=1e-13, max_iterations=100000)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        u, _ = p.solve(opts)
        _, dc = p.compliance()
        F = p.output_derivative(M.OUTPUT_COMPLIANCE, u)
        for e in (0, 17, 53):
            du = p.sensitivity_solve(u, M.PARAM_DENSITY, e, opts)
            assert abs(F @ du - dc[e]) <= 1e-9 * abs(dc[e])
        h = 1e-5
        e = 17
        du = p.sensitivity_solve(u, M.PARAM_DENSITY, e, opts)
        r2 = rho.copy()
        r2[e] += h
        p.set_design(r2)
        up, _ = p.solve(opts)
        r2[e] -= 2 * h
        p.set_design(r2)
        um, _ = p.solve(opts)
    assert rel((up - um) / (2 * h), du) < 1e-6


def test_element_calculations_at_a_local_solution():
    """The per-element plugin call (elem_calculations after set_elem_solution) on the
    element-local solution against the oracle element, and its density sensitivity."""
    coords, conn = distorted_hex8()
    rng = np.random.default_rng(4)
    rho = rng.uniform(0.1, 1.0, conn.shape[0])
    with M.Problem(M.PHYS_HEX8, coords, conn, M.SIMP_MATERIAL) as p:
        p.set_design(rho)
        d = O.simp_desc(1, 1, 1)
        E, dE = O.simp_modulus(d, rho)
        for e in range(conn.shape[0]):
            ue = rng.standard_normal(24)
            f, K = p.element_calculations(e, ue)
            f_ref, K_ref = O.hex8_internal(coords[conn[e]], E[e], 0.3, ue)
            assert rel(K, K_ref) < RTOL_ELEM and rel(f, f_ref) < RTOL_ELEM
            df = p.element_sensitivity(e, ue, M.PARAM_DENSITY, e)
            assert rel(df, O.hex8_internal_sens(coords[conn[e]], dE[e], 0.3, ue)) < RTOL_ELEM
            other = p.element_sensitivity(e, ue, M.PARAM_DENSITY, (e + 1) % conn.shape[0])
            assert np.all(other == 0.0)


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
