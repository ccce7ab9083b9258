"""The oracle's stress output (StructuralElement3D::calculate_stress,
src/elasticity/solid_element_3d.cpp:1147-1270; von Mises of
StressStrainOutputBase::Data, stress_output_base.cpp:183-271) and its KS aggregate
with the adjoint sensitivity of example_6 (ks_stress_output.cpp:41-246,
examples/structural/example_6/example_6.cpp:798-874), pinned by closed-form
stresses, finite differences and the KS bound."""
import numpy as np
import pytest

import oracle as O


def brick(distort=0.0, seed=0):
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float) * [1.2, 0.9, 1.1]
    return X + distort * np.random.default_rng(seed).uniform(-1, 1, X.shape)


def var_blocked(disp):
    return np.ascontiguousarray(disp.T.reshape(24))


def test_homogeneous_strain_gives_the_closed_form_stress():
    E, nu = 70.0, 0.3
    X = brick(0.1)
    G = E / (2 * (1 + nu))
    tau = 1e-3
    # pure shear gamma_xy: u = gamma y, sigma_xy = G gamma, von Mises sqrt(3) tau
    gamma = tau / G
    disp = np.zeros((8, 3))
    disp[:, 0] = gamma * X[:, 1]
    sig, vm, jxw, _ = O.hex8_stress(X, E, nu, var_blocked(disp))
    assert np.allclose(sig[:, 3], tau, rtol=1e-12) and np.abs(sig[:, [0, 1, 2, 4, 5]]).max() < 1e-15
    assert np.allclose(vm, np.sqrt(3) * tau, rtol=1e-12)
    # uniaxial stress: eps_xx = s/E, eps_yy = eps_zz = -nu s/E, von Mises = s
    s = 2e-3
    disp = np.stack([s / E * X[:, 0], -nu * s / E * X[:, 1], -nu * s / E * X[:, 2]], axis=1)
    sig, vm, jxw, _ = O.hex8_stress(X, E, nu, var_blocked(disp))
    assert np.allclose(sig[:, 0], s, rtol=1e-12) and np.allclose(vm, s, rtol=1e-12)
    jxw = O.hex8_stress(brick(), E, nu, var_blocked(disp))[2]
    assert abs(jxw.sum() - 1.2 * 0.9 * 1.1) < 1e-14  # sum of JxW = the brick's volume


@pytest.mark.parametrize("nonlinear", [False, True])
def test_stress_derivative_is_the_finite_difference(nonlinear):
    X = brick(0.1, seed=2)
    u = np.random.default_rng(3).normal(scale=0.05, size=24)
    sig, vm, jxw, ds = O.hex8_stress(X, 5.0, 0.3, u, nonlinear, True)
    h = 1e-6
    for c in range(24):
        up, um = u.copy(), u.copy()
        up[c] += h
        um[c] -= h
        fd = (O.hex8_stress(X, 5.0, 0.3, up, nonlinear)[0] - O.hex8_stress(X, 5.0, 0.3, um, nonlinear)[0]) / (2 * h)
        assert np.abs(ds[:, :, c] - fd).max() <= 1e-7 * np.abs(ds).max()


def cantilever(nx=4, ny=2, nz=2, load=1.0):
    coords, conn = O.grid_hex8(nx, ny, nz)
    nn = coords.shape[0]
    fixed = np.zeros(nn * 3, np.uint8)
    fixed[(np.where(coords[:, 0] == 0)[0][:, None] * 3 + np.arange(3)).reshape(-1)] = 1
    F = np.zeros(nn * 3)
    tip = np.where((coords[:, 0] == nx) & (coords[:, 2] == 0))[0]
    F[tip * 3 + 2] = -load / tip.shape[0]
    return coords, conn, fixed, F


def simp(rho, penal, E0=1.0, Emin=1e-9):
    rmin = Emin / E0
    return E0 * (rmin + (1 - rmin) * rho ** penal), E0 * (1 - rmin) * penal * rho ** (penal - 1)


@pytest.mark.parametrize("nonlinear", [False, True])
def test_ks_adjoint_sensitivity_matches_finite_differences(nonlinear):
    coords, conn, fixed, F = cantilever(3, 1, 1, load=0.02 if nonlinear else 1.0)
    rho = np.array([0.9, 0.6, 0.8])
    p_ks, s0 = 8.0, 0.5

    def q_of(r):
        E, _ = simp(r, 3.0)
        Es, _ = simp(r, 0.5)
        if nonlinear:
            u, _ = O.newton_hex8_gl(coords, conn, E, 0.3, F, fixed, rtol=1e-14)
        else:
            rp, cl = O.csr_pattern(conn, coords.shape[0], 3)
            u, _, _ = O.pcg(rp, cl, O.assemble_hex8(coords, conn, E, 0.3, rp, cl, fixed), F, 1e-15, 100000)
        return u, O.ks_stress(coords, conn, Es, simp(r, 0.5)[1], 0.3, u, p_ks, s0, nonlinear)[0]

    u, q0 = q_of(rho)
    E, dE = simp(rho, 3.0)
    Es, dEs = simp(rho, 0.5)
    q, vmax, total = O.ks_stress_total_sensitivity(coords, conn, E, dE, Es, dEs, 0.3, u, fixed, p_ks,
                                                   s0, nonlinear)
    assert abs(q - q0) < 1e-14
    h = 1e-6
    for e in range(3):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (q_of(rp)[1] - q_of(rm)[1]) / (2 * h)
        assert abs(total[e] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(total).max())


def test_ks_is_a_lower_bound_that_approaches_the_maximum():
    coords, conn, fixed, F = cantilever()
    E = np.full(conn.shape[0], 1.0)
    rp, cl = O.csr_pattern(conn, coords.shape[0], 3)
    u, _, _ = O.pcg(rp, cl, O.assemble_hex8(coords, conn, E, 0.3, rp, cl, fixed), F, 1e-14, 100000)
    s0 = 1.0
    qs = []
    for p in (4.0, 32.0, 256.0):
        q, vmax, _, _ = O.ks_stress(coords, conn, E, np.zeros_like(E), 0.3, u, p, s0)
        assert q <= (vmax - s0) / s0 + 1e-12
        qs.append(q)
    assert qs[0] < qs[1] < qs[2]
    assert abs(qs[2] - (vmax - s0) / s0) < 0.05 * abs(vmax)


# ---------------------------------------------------------------- device source on the host
def _host_stress():
    import ctypes
    import os
    import subprocess
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = os.path.join(repo, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libstress_element_host.so")
    src = os.path.join(repo, "tests", "cpp", "stress_element_host.cpp")
    hdr = os.path.join(repo, "mast-multiphysics_gb300", "csrc", "hex8_gl.cuh")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                            "-x", "c++", "-I", os.path.dirname(hdr), src, "-o", so],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    d = ctypes.c_double
    L.stress_element_host.argtypes = [p, d, d, p, ctypes.c_int, d, d, p, p, p, p]
    return L


@pytest.mark.parametrize("nonlinear,scale", [(False, 1e-3), (True, 0.05), (False, 1e-9), (True, 1e-9)])
def test_device_stress_source_matches_the_oracle(nonlinear, scale):
    """The stress phases of the CUDA kernel (hex8_gl.cuh), lane by lane on the host, against
    the oracle's B-operator form: von Mises, JxW, the KS exponential and its u-gradient."""
    L = _host_stress()
    X = brick(0.1, seed=7)
    u = np.random.default_rng(8).normal(scale=scale, size=24)
    p_ks, s0 = 6.0, 0.7 * scale
    vm, jxw, ex, g = np.zeros(8), np.zeros(8), np.zeros(8), np.zeros(24)
    assert L.stress_element_host(np.ascontiguousarray(X.reshape(24)), 2.0, 0.3, u, int(nonlinear), p_ks,
                                 s0, vm, jxw, ex, g) == 0
    sig, vmo, jxwo, ds = O.hex8_stress(X, 2.0, 0.3, u, nonlinear, True)
    assert np.abs(vm - vmo).max() <= 1e-12 * vmo.max()
    assert np.abs(jxw - jxwo).max() <= 1e-14
    exo = np.exp(p_ks * (vmo - s0) / s0)
    assert np.abs(ex - exo).max() <= 1e-11 * exo.max()
    go = sum((O._dvm_dsig(sig[q]) @ ds[q]) * exo[q] * jxwo[q] for q in range(8))
    assert np.abs(g - go).max() <= 1e-11 * np.abs(go).max()
