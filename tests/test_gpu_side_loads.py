"""Side loads (mg_set_side_loads) through the C ABI against the FP64 oracle: HEX8 face
pressure in the linear solve (plain and mixed forms) and the QUAD4 heat-flux residual."""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def cantilever_arrays(nx, ny, nz, load):
    """mesh, Dirichlet mask and point loads of mastgpu.simp_cantilever"""
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


def pressure_loads(coords, conn, nx, nz):
    """-0.3 on the top faces (side 5) of the top layer, +0.2 on the x = max faces (side 2)"""
    cz = coords[conn].mean(axis=1)
    top = np.where(cz[:, 2] > nz - 1)[0]
    end = np.where(cz[:, 0] > nx - 1)[0]
    elems = np.concatenate([top, end]).astype(np.int32)
    sides = np.concatenate([np.full(top.shape, 5), np.full(end.shape, 2)]).astype(np.int32)
    vals = np.concatenate([np.full(top.shape, -0.3), np.full(end.shape, 0.2)])
    return elems, sides, vals


def oracle_load(coords, conn, elems, sides, vals, F_point, fixed):
    F = F_point.copy()
    for e, s, v in zip(elems, sides, vals):
        f = O.hex8_pressure(coords[conn[e]], int(s), float(v)).reshape(3, 8).T  # (node, comp)
        for a in range(8):
            F[conn[e][a] * 3:conn[e][a] * 3 + 3] += f[a]
    F[fixed == 1] = 0.0
    return F


def test_face_pressure_solve_matches_oracle():
    nx, ny, nz = 16, 8, 8
    coords, conn, fixed, Fp = cantilever_arrays(nx, ny, nz, 1.0)
    elems, sides, vals = pressure_loads(coords, conn, nx, nz)
    F = oracle_load(coords, conn, elems, sides, vals, Fp, fixed)
    rp, cl = O.csr_pattern(conn, coords.shape[0], 3)
    K = O.assemble_hex8(coords, conn, np.ones(conn.shape[0]), 0.3, rp, cl, fixed)
    u_ref, _, _ = O.pcg(rp, cl, K, F, 1e-15, 100000)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_side_loads(elems, sides, vals)
        u, rep = p.solve(M.default_opts(rtol=1e-12))
        c, _ = p.compliance(want_sens=False)
        # the mixed form rebuilds its load vector from the side loads
        um, repm = p.solve(M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3))
        # clearing the side loads leaves the point loads
        p.set_side_loads([], [], [])
        u0, _ = p.solve(M.default_opts(rtol=1e-12))
    assert rel(u, u_ref) < 1e-10
    assert abs(c - F @ u_ref) <= 1e-10 * abs(F @ u_ref)
    assert abs(F @ um - F @ u_ref) <= 1e-6 * abs(F @ u_ref)  # as the other mixed-form tests
    u0_ref, _, _ = O.pcg(rp, cl, K, Fp, 1e-15, 100000)
    assert rel(u0, u0_ref) < 1e-10


def test_heat_flux_residual_matches_oracle():
    n = 8
    with M.heat_square(n, n) as p:
        top = (np.arange(n) + n * (n - 1)).astype(np.int32)
        p.set_side_loads(top, np.full(n, 2, np.int32), np.full(n, 0.7))
        T = np.random.default_rng(3).uniform(0.0, 2.0, p.n_dofs)
        fixed = np.zeros(p.n_dofs, np.uint8)
        fixed[(n + 1) * np.arange(n + 1)] = 1
        T[fixed == 1] = 0.0
        R = p.residual_and_jacobian(T, want_J=False)
    coords, conn = O.grid_quad4(n, n)
    rp, cl = O.csr_pattern(conn, coords.shape[0], 1)
    conv_e = (n - 1) + n * np.arange(n)
    src = O.heat_source_field(n, n)
    _, R_ref = O.assemble_quad4_heat(coords, conn, 1.0, 0.01, None, 1.0, src, conv_e.astype(np.int32),
                                     np.ones(n, np.int32), 10.0, 0.0, T, True, rp, cl, fixed)
    for e in top:
        f = O.quad4_heat_flux(coords[conn[e]], 2, 0.7, 1.0)
        for a in range(4):
            if not fixed[conn[e][a]]:
                R_ref[conn[e][a]] += f[a]
    assert rel(R, R_ref) < 1e-12


def test_side_loads_reject_bad_input_and_the_membrane():
    with M.simp_cantilever(2, 1, 1) as p:
        for e, s, v in ((5, 0, 1.0), (0, 6, 1.0), (0, 0, np.nan), (-1, 0, 1.0)):
            with pytest.raises(M.MastGpuError) as err:
                p.set_side_loads([e], [s], [v])
            assert err.value.status == M.MG_EINVAL
    coords, conn = M.grid_quad4(2, 2)
    with M.Problem(M.PHYS_MEMBRANE, coords, conn, M.SIMP_MATERIAL) as p:
        with pytest.raises(M.MastGpuError) as err:
            p.set_side_loads([0], [0], [1.0])
        assert err.value.status == M.MG_ENOTSUP
