"""Mixed-precision matrix-free SIMP form (tcgen05 TF32 / BF16 operator, FP32
inner CG, FP64 refinement) against the FP64 oracle.

Accuracy bar: FP64 outer residual ||f - K u|| / ||f|| <= 1e-8 and at most 1e-6
relative error in compliance and sensitivities against the FP64 oracle.
Operator check: one application against the FP64 CSR product, relative error
below the input rounding of the format (TF32 2^-11, BF16 2^-8) times a small
factor.
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu

TOL_OP = {M.MIXED_TF32: 4e-3, M.MIXED_BF16: 3e-2, M.MIXED_TF32X3: 2e-5, M.MIXED_BF16X3: 2e-4,
          M.OPERATOR_FACTORED_FP32: 2e-6}
ALL = [M.MIXED_TF32, M.MIXED_BF16, M.MIXED_TF32X3, M.MIXED_BF16X3]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.parametrize("shape", [(8, 4, 4), (16, 8, 8), (12, 7, 5), (17, 9, 3), (40, 9, 10)])
def test_factored_level_operator_matches_fp64_csr(shape):
    """The multigrid level operator (FP32, CUDA cores, factored element
    stiffness; tiles of 31 x 7 owned nodes, so the 40 x 9 grid spans several)
    against the FP64 CSR product: FP32 rounding only."""
    nx, ny, nz = shape
    rng = np.random.default_rng(2)
    rho = rng.uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        x = rng.standard_normal(p.n_dofs)
        fixed = O.simp_fixed_mask(O.simp_desc(nx, ny, nz))
        x[fixed == 1] = 0.0
        p.residual_and_jacobian(np.zeros(p.n_dofs), want_R=False)
        y_ref = p.spmv(x)
        y = p.matfree_apply(x, M.OPERATOR_FACTORED_FP32)
    y_ref[fixed == 1] = 0.0
    assert rel(y, y_ref) < TOL_OP[M.OPERATOR_FACTORED_FP32]
    assert np.all(y[fixed == 1] == 0.0)


@pytest.mark.parametrize("smoother", [M.SMOOTHER_FACTORED, M.SMOOTHER_TENSOR])
def test_both_smoother_operators_converge(smoother):
    nx, ny, nz = 32, 16, 16
    rho = np.random.default_rng(7).uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        _, rep = p.solve(M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3,
                                        smoother_operator=smoother))
        c, dc = p.compliance()
    assert rep.status == 0 and rep.relres <= 1e-8, (rep.status, rep.relres)
    _, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-12, maxit=10 ** 6), rho)
    assert abs(c - r.compliance) / r.compliance < 1e-6
    assert np.abs(dc - dc_ref).max() / np.abs(dc_ref).max() < 1e-6


@pytest.mark.parametrize("prec", ALL)
@pytest.mark.parametrize("shape", [(8, 4, 4), (16, 8, 8), (12, 7, 5), (17, 9, 3)])
def test_operator_matches_fp64_csr(prec, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(1)
    rho = rng.uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        x = rng.standard_normal(p.n_dofs)
        fixed = O.simp_fixed_mask(O.simp_desc(nx, ny, nz))
        x[fixed == 1] = 0.0
        p.residual_and_jacobian(np.zeros(p.n_dofs), want_R=False)
        y_ref = p.spmv(x)
        y = p.matfree_apply(x, prec)
    y_ref[fixed == 1] = 0.0
    assert rel(y, y_ref) < TOL_OP[prec]


@pytest.mark.parametrize("prec", ALL + [M.OPERATOR_FACTORED_FP32])
def test_operator_matches_oracle_assembly(prec):
    """One application of each matrix-free operator against the oracle's own FP64
    assembly (O.assemble_hex8, the restated element loop) and CSR product, with no
    GPU CSR in between."""
    nx, ny, nz = 12, 7, 5
    rng = np.random.default_rng(12)
    rho = rng.uniform(0.01, 1.0, nx * ny * nz)
    d = O.simp_desc(nx, ny, nz)
    fixed = O.simp_fixed_mask(d)
    x = rng.standard_normal(3 * (nx + 1) * (ny + 1) * (nz + 1))
    x[fixed == 1] = 0.0
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        y = p.matfree_apply(x, prec)
    coords, conn = O.grid_hex8(nx, ny, nz)
    rp, cols = O.csr_pattern(conn, coords.shape[0], 3)
    E, _ = O.simp_modulus(d, rho)
    vals = O.assemble_hex8(coords, conn, E, 0.3, rp, cols, fixed)
    y_ref = O.spmv(rp, cols, vals, x)
    y_ref[fixed == 1] = 0.0
    assert rel(y, y_ref) < TOL_OP[prec]
    assert np.all(y[fixed == 1] == 0.0)


@pytest.mark.parametrize("pc", [M.PC_MULTIGRID, M.PC_JACOBI])
@pytest.mark.parametrize("prec", [M.MIXED_TF32, M.MIXED_TF32X3, M.MIXED_BF16X3])
def test_mixed_solve_matches_oracle(prec, pc):
    nx, ny, nz = 16, 8, 8
    rho = np.random.default_rng(3).uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(precision=prec, rtol=1e-8, inner_rtol=1e-3,
                                        preconditioner=pc))
        c, dc = p.compliance()
    assert rep.status == 0 and rep.relres <= 1e-8, (rep.status, rep.relres)
    _, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-12, maxit=10 ** 6), rho)
    assert abs(c - r.compliance) / r.compliance < 1e-6
    assert np.abs(dc - dc_ref).max() / np.abs(dc_ref).max() < 1e-6


def test_mixed_solve_is_deterministic():
    nx, ny, nz = 16, 8, 8
    rho = np.random.default_rng(4).uniform(0.01, 1.0, nx * ny * nz)
    outs = []
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        for _ in range(2):
            u, rep = p.solve(M.default_opts(precision=M.MIXED_TF32, rtol=1e-8))
            outs.append((u, rep.krylov_iterations))
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]


def test_single_pass_bf16_reports_its_limit():
    """One BF16 product per element (8-bit operand mantissa) stalls the FP64
    refinement on this contrast (1e6); the solve must end with MG_ENOCONV and a
    finite residual, never a hang or NaN.  MIXED_BF16X3 is the BF16 variant
    that reaches 1e-8."""
    nx, ny, nz = 16, 8, 8
    rho = np.random.default_rng(3).uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        _, rep = p.solve(M.default_opts(precision=M.MIXED_BF16, rtol=1e-8, max_refinements=8,
                                        preconditioner=M.PC_JACOBI), raise_on_error=False)
    assert rep.status in (M.MG_OK, M.MG_ENOCONV) and np.isfinite(rep.relres)


@pytest.mark.parametrize("shape", [(32, 16, 16), (24, 12, 8)])
def test_multigrid_cuts_iterations(shape):
    """The multigrid V-cycle (Chebyshev-Jacobi smoothers, rediscretised coarse
    grids) preconditions the same FP32 CG: same answer, far fewer iterations."""
    nx, ny, nz = shape
    rho = np.random.default_rng(6).uniform(0.01, 1.0, nx * ny * nz)
    out = {}
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        for pc in (M.PC_JACOBI, M.PC_MULTIGRID):
            u, rep = p.solve(M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, preconditioner=pc))
            c, _ = p.compliance(want_sens=False)
            out[pc] = (rep.krylov_iterations, c, rep.relres)
    assert out[M.PC_MULTIGRID][2] <= 1e-8 and out[M.PC_JACOBI][2] <= 1e-8
    assert abs(out[M.PC_MULTIGRID][1] - out[M.PC_JACOBI][1]) / out[M.PC_JACOBI][1] < 1e-7
    assert out[M.PC_MULTIGRID][0] * 4 < out[M.PC_JACOBI][0]


def test_outer_residual_matches_the_fp64_csr_residual():
    """The refinement's outer residual r = f - K u is formed on FP64 data with the
    element products in double-float arithmetic (48-bit significand); the relative
    residual it reports must agree with the plain FP64 CSR residual of the same u
    to far below the 1e-8 target (absolute 1e-11 in units of ||f||)."""
    nx, ny, nz = 32, 16, 16
    rho = np.random.default_rng(8).uniform(0.01, 1.0, nx * ny * nz)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-2))
        F = -p.residual_and_jacobian(np.zeros(p.n_dofs), want_J=False)
        R = p.residual_and_jacobian(u, want_J=False)
    true_relres = np.linalg.norm(R) / np.linalg.norm(F)
    assert rep.status == 0 and rep.relres <= 1e-8
    assert abs(rep.relres - true_relres) <= 1e-11, (rep.relres, true_relres)


@pytest.mark.parametrize("shape", [(32, 16, 16), (20, 10, 10)])
def test_cluster_bottom_vcycle_matches_the_one_cta_form(shape):
    """A single-design solve runs the small multigrid levels on a thread-block
    cluster (from the first level below the design with at most 4,096 nodes: the
    whole chain 16x8x8 .. 4x2x2 of the 32x16x16 design); a batch runs them in one
    CTA from the first level with at most 1,024 nodes and the rest level by level.
    Both are the same V-cycle up to FP32 rounding: the same iteration count within
    one, and results that match each other and the FP64 oracle.  (20x10x10 has a
    single coarse level, 10x5x5, smoothed rather than solved directly.)"""
    nx, ny, nz = shape
    rho = np.random.default_rng(11).uniform(0.01, 1.0, nx * ny * nz)
    o = M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=300.0)
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(rho)
        _, rep = p.solve(o)
        c, dc = p.compliance()
    with M.Batch([dict(nx=nx, ny=ny, nz=nz, rho=rho, spans=[(0, ny)])]) as b:
        rc, reps = b.solve(o)
        cb, dcb, _ = b.results(0)
    assert rep.status == 0 and rep.relres <= 1e-8
    assert rc == 0 and reps[0].status == 0 and reps[0].relres <= 1e-8
    assert abs(rep.krylov_iterations - reps[0].krylov_iterations) <= 1, \
        (rep.krylov_iterations, reps[0].krylov_iterations)
    assert abs(c - cb[0]) / abs(cb[0]) < 1e-8
    assert np.abs(dc - dcb[0]).max() / np.abs(dcb[0]).max() < 1e-7
    _, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-12, maxit=10 ** 6), rho)
    assert abs(c - r.compliance) / r.compliance < 1e-6
    assert np.abs(dc - dc_ref).max() / np.abs(dc_ref).max() < 1e-6


def test_cluster_bottom_result_does_not_depend_on_the_cluster_size(monkeypatch):
    """Every dof of the cluster V-cycle is computed by one thread in a fixed order,
    whichever CTA owns it: 16, 4 and 1 CTA per chain give bitwise the same solve."""
    nx, ny, nz = 32, 16, 16
    rho = np.random.default_rng(13).uniform(0.01, 1.0, nx * ny * nz)
    o = M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=300.0)
    out = []
    for cs in ("16", "4", "1"):
        monkeypatch.setenv("MASTGPU_BOTTOM_CLUSTER", cs)
        with M.simp_cantilever(nx, ny, nz) as p:
            p.set_design(rho)
            u, rep = p.solve(o)
        assert rep.status == 0 and rep.relres <= 1e-8
        out.append((u, rep.krylov_iterations))
    for u, its in out[1:]:
        assert its == out[0][1] and np.array_equal(u, out[0][0])
