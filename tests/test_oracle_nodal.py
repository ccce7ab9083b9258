"""Nodal density field (MAST example 6 reads its SIMP density through a
MeshFieldFunction over a FIRST-order LAGRANGE "rho" variable,
examples/structural/example_6/example_6.cpp:104-137, 250-252): the modulus is
evaluated at each Gauss point from the trilinear density there.  The oracle's
nodal path is pinned here by its own identities (uniform field = element field,
per-point moduli = one modulus) and by central differences of the compliance."""
import numpy as np
import pytest

import oracle as O


def test_per_point_moduli_reduce_to_one_modulus():
    rng = np.random.default_rng(0)
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                 float) * [1.0, 0.7, 1.3] + 0.05 * rng.standard_normal((8, 3))
    u = rng.standard_normal(24)
    f1, K1 = O.hex8_internal(X.ravel(), 2.5, 0.3, u)
    f2, K2 = O.hex8_internal_qp(X.ravel(), np.full(8, 2.5), 0.3, u)
    assert np.allclose(K1, K2, rtol=0, atol=1e-13 * np.abs(K1).max())
    assert np.allclose(f1, f2, rtol=0, atol=1e-13 * np.abs(f1).max())
    # linear in the per-point moduli: K(Eq) = sum_q Eq_q K(e_q)
    Eq = rng.uniform(0.5, 2.0, 8)
    _, K = O.hex8_internal_qp(X.ravel(), Eq, 0.3, u)
    Ks = sum(Eq[q] * O.hex8_internal_qp(X.ravel(), np.eye(8)[q], 0.3, u)[1] for q in range(8))
    assert np.abs(K - Ks).max() <= 1e-13 * np.abs(K).max()


def test_uniform_nodal_field_equals_the_element_field():
    nx, ny, nz = 6, 3, 3
    desc = O.simp_desc(nx, ny, nz, rtol=1e-13, maxit=10 ** 5)
    c = 0.6
    u_e, dc_e, r_e = O.simp_solve(desc, np.full(nx * ny * nz, c))
    u_n, dc_n, r_n = O.simp_solve_nodal(desc, np.full((nx + 1) * (ny + 1) * (nz + 1), c))
    assert np.linalg.norm(u_n - u_e) <= 1e-11 * np.linalg.norm(u_e)
    assert abs(r_n.compliance - r_e.compliance) <= 1e-12 * r_e.compliance
    # a uniform change of the field moves every element density alike
    assert abs(dc_n.sum() - dc_e.sum()) <= 1e-10 * abs(dc_e.sum())


def test_nodal_sensitivity_matches_central_differences():
    nx, ny, nz = 4, 2, 2
    desc = O.simp_desc(nx, ny, nz, rtol=1e-14, maxit=10 ** 5)
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    rho = np.random.default_rng(3).uniform(0.3, 1.0, nn)
    _, dc, _ = O.simp_solve_nodal(desc, rho)
    h = 1e-6
    for n in (0, 7, 22, 31, nn - 1):
        rp, rm = rho.copy(), rho.copy()
        rp[n] += h
        rm[n] -= h
        cp = O.simp_solve_nodal(desc, rp, want_sens=False)[2].compliance
        cm = O.simp_solve_nodal(desc, rm, want_sens=False)[2].compliance
        fd = (cp - cm) / (2 * h)
        assert abs(fd - dc[n]) <= 1e-6 * np.abs(dc).max(), (n, fd, dc[n])
