"""Density filter of MAST::FilterBase (src/level_set/filter_base.cpp:58-95,
:275-359, :378-437): normalised hat weights (r - d) over the points within r,
non-design points passed through, and its transpose (the design-gradient chain
rule).  The oracle (O(n^2) search, as the reference's `_init`) is checked
first; the GPU stencil and CSR forms are compared with it."""
import numpy as np
import pytest

import mastgpu as M
import oracle as O


def test_oracle_filter_hand_case_on_a_line():
    # three points 1 apart, r = 1.5: point 0 sees itself (weight 1.5) and point 1
    # (0.5), so w = (0.75, 0.25); point 1 sees all three: (0.5, 1.5, 0.5) / 2.5
    xyz = np.array([[0.0], [1.0], [2.0]])
    x = np.array([1.0, 2.0, 4.0])
    y = O.filter_points(xyz, 1.5, x)
    assert np.allclose(y, [0.75 * 1 + 0.25 * 2, (0.5 * 1 + 1.5 * 2 + 0.5 * 4) / 2.5, 0.25 * 2 + 0.75 * 4],
                       rtol=1e-15)
    # a point at exactly r contributes weight r - d = 0
    y2 = O.filter_points(xyz, 1.0, x)
    assert np.allclose(y2, x)


def test_oracle_filter_properties():
    xyz = O.grid_centroids(7, 5, 4)
    rng = np.random.default_rng(0)
    x = rng.uniform(0.01, 1.0, len(xyz))
    g = rng.normal(size=len(xyz))
    for r in (1.2, 2.1):
        assert np.allclose(O.filter_points(xyz, r, np.ones(len(xyz))), 1.0, rtol=1e-14)  # partition of unity
        y = O.filter_points(xyz, r, x)
        assert abs(y @ g - x @ O.filter_points(xyz, r, g, transpose=True)) < 1e-12 * abs(y @ g)
        dv = (np.arange(len(xyz)) % 4 != 0).astype(np.uint8)
        yd = O.filter_points(xyz, r, x, dv)
        assert np.array_equal(yd[dv == 0], x[dv == 0])
        assert abs(yd @ g - x @ O.filter_points(xyz, r, g, dv, transpose=True)) < 1e-12 * abs(yd @ g)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(10, 6, 5), (9, 7, 0)])
@pytest.mark.parametrize("radius", [1.5, 2.3])
@pytest.mark.parametrize("masked", [False, True])
def test_grid_filter_matches_oracle(dims, radius, masked):
    nx, ny, nz = dims
    xyz = O.grid_centroids(nx, ny, nz)
    n = len(xyz)
    rng = np.random.default_rng(1)
    x = rng.uniform(0.01, 1.0, n)
    g = rng.normal(size=n)
    dv = (rng.uniform(size=n) > 0.2).astype(np.uint8) if masked else None
    with M.Filter.grid(nx, ny, nz, radius, dv=dv) as f:
        y = f.apply(x)
        yt = f.apply(g, transpose=True)
    assert rel(y, O.filter_points(xyz, radius, x, dv)) < 1e-13
    assert rel(yt, O.filter_points(xyz, radius, g, dv, transpose=True)) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("masked", [False, True])
def test_points_filter_matches_oracle(masked):
    rng = np.random.default_rng(2)
    xyz = rng.uniform(0.0, 1.0, (600, 3))
    x = rng.uniform(0.01, 1.0, 600)
    g = rng.normal(size=600)
    dv = (rng.uniform(size=600) > 0.3).astype(np.uint8) if masked else None
    with M.Filter(xyz, 0.22, dv=dv) as f:
        assert rel(f.apply(x), O.filter_points(xyz, 0.22, x, dv)) < 1e-13
        assert rel(f.apply(g, transpose=True), O.filter_points(xyz, 0.22, g, dv, transpose=True)) < 1e-13


@pytest.mark.gpu
def test_filtered_compliance_gradient_matches_fd():
    """C(rho) = compliance at the filtered densities F rho: dC/drho = F^T dC/drho_f,
    checked against central differences of the plain FP64 solve."""
    nx, ny, nz = 8, 4, 4
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.2, 0.9, nx * ny * nz)
    opts = M.default_opts(precision=M.PLAIN_FP64, rtol=1e-12)
    with M.Filter.grid(nx, ny, nz, 1.6) as f, M.simp_cantilever(nx, ny, nz) as p:
        def C(r):
            p.set_design(f.apply(r))
            p.solve(opts)
            c, dc = p.compliance()
            return c, dc
        c0, dc_f = C(rho)
        grad = f.apply(dc_f, transpose=True)
        for e in (0, 37, 100):
            h = 1e-5
            rp, rm = rho.copy(), rho.copy()
            rp[e] += h
            rm[e] -= h
            fd = (C(rp)[0] - C(rm)[0]) / (2 * h)
            assert abs(fd - grad[e]) <= 1e-6 * abs(grad[e]) + 1e-12, (e, fd, grad[e])
