"""The precision workload at its full size: HEX8 SIMP cantilever 128x64x64
(524,288 elements, 1,635,075 dofs), densities U[0.01, 1] from default_rng(0).

The mixed-precision form (tensor-core split-TF32 and split-BF16 operators, FP32
multigrid-preconditioned CG, FP64 refinement to a 1e-8 relative FP64 residual)
against the oracle's FP64 fixture (tests/golden/simp_128x64x64_seed0.npz: compliance
and dC/drho of a 1e-11 Jacobi-PCG solve, stored in FP64): at most 1e-6 relative
error in compliance and sensitivities (max-norm relative for dC/drho).
"""
import os

import numpy as np
import pytest

import mastgpu as M

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

HERE = os.path.dirname(os.path.abspath(__file__))
NX, NY, NZ = 128, 64, 64
TOL = 1e-6


@pytest.fixture(scope="module")
def problem():
    g = np.load(os.path.join(HERE, "golden", "simp_128x64x64_seed0.npz"))
    assert g["dc"].dtype == np.float64
    rho = np.random.default_rng(0).uniform(0.01, 1.0, NX * NY * NZ)
    p = M.simp_cantilever(NX, NY, NZ)
    p.set_design(rho)
    yield p, g, rho
    p.close()


@pytest.mark.parametrize("prec", [M.MIXED_TF32X3, M.MIXED_BF16X3])
def test_full_size_mixed_solve_matches_the_fp64_fixture(problem, prec):
    p, g, rho = problem
    p.set_design(rho)
    u, rep = p.solve(M.default_opts(precision=prec, rtol=1e-8, inner_rtol=1e-3, timeout_s=300.0))
    c, dc = p.compliance()
    assert rep.status == 0 and rep.relres <= 1e-8, (rep.status, rep.relres)
    c_ref = float(g["compliance"])
    assert abs(c - c_ref) <= TOL * abs(c_ref), (c, c_ref)
    err = np.abs(dc - g["dc"]).max() / np.abs(g["dc"]).max()
    assert err <= TOL, err
    # the tip deflection of the fixture (node (nx, 0, 0), z component)
    assert abs(u[NX * 3 + 2] - float(g["u_tip"])) <= 1e-6 * abs(float(g["u_tip"]))
