"""Side loads: HEX8 surface pressure (StructuralElement3D::surface_pressure_residual,
src/elasticity/solid_element_3d.cpp:815-876) and QUAD4 heat flux
(HeatConductionElementBase::surface_flux_residual,
src/heat_conduction/heat_conduction_elem_base.cpp:876-913).  The oracle is pinned by
exact integrals (a bilinear face's vector area, the edge length, the first moment), and
the device source (side_loads.cuh, a different but equivalent form: Nanson's relation on
the reference cube) is compared with it on the host."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# libMesh Hex8 side -> nodes, and each side's outward reference normal
SIDE_NODES = [(0, 3, 2, 1), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]
SIDE_NORMAL = [(0, 0, -1), (0, -1, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, 0, 1)]


def brick(distort=0.0, seed=0):
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float) * [2.0, 1.5, 0.5]
    return X + distort * np.random.default_rng(seed).uniform(-1, 1, X.shape)


@pytest.mark.parametrize("side", range(6))
def test_pressure_on_a_box_face_is_p_area_n_shared_by_its_nodes(side):
    X = brick()
    f = O.hex8_pressure(X, side, 3.0).reshape(3, 8).T  # (node, component)
    dims = np.array([2.0, 1.5, 0.5])
    n = np.array(SIDE_NORMAL[side], dtype=float)
    area = np.prod(dims[n == 0])
    for a in range(8):
        expect = 3.0 * area / 4 * n if a in SIDE_NODES[side] else np.zeros(3)
        assert np.allclose(f[a], expect, atol=1e-14)


@pytest.mark.parametrize("side", range(6))
def test_pressure_resultant_is_p_times_the_vector_area(side):
    """For a bilinear face the vector area int n dA is (x2 - x0) x (x3 - x1) / 2."""
    X = brick(0.15, seed=side)
    f = O.hex8_pressure(X, side, 1.7).reshape(3, 8).T
    q = [X[i] for i in SIDE_NODES[side]]
    vec_area = 0.5 * np.cross(q[2] - q[0], q[3] - q[1])
    assert np.allclose(f.sum(axis=0), 1.7 * vec_area, rtol=1e-13, atol=1e-14)
    # outward: the resultant points away from the element centroid
    assert np.dot(f.sum(axis=0), np.mean(q, axis=0) - X.mean(axis=0)) > 0


@pytest.mark.parametrize("side", range(4))
def test_heat_flux_on_an_edge_is_half_the_edge_flux_per_node(side):
    X = np.array([[0.0, 0.0], [2.0, 0.2], [2.3, 1.4], [-0.1, 1.0]])
    f = O.quad4_heat_flux(X, side, 5.0, 0.3)
    a0, a1 = side, (side + 1) % 4
    L = np.linalg.norm(X[a1] - X[a0])
    expect = np.zeros(4)
    expect[[a0, a1]] = 5.0 * 0.3 * L / 2
    assert np.allclose(f, expect, rtol=1e-14)


def _host():
    out = os.path.join(REPO, "tests", "cpp", "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libside_loads_host.so")
    src = os.path.join(REPO, "tests", "cpp", "side_loads_host.cpp")
    hdr = os.path.join(REPO, "mast-multiphysics_gb300", "csrc", "side_loads.cuh")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-x", "c++", "-I",
                            os.path.dirname(hdr), src, "-o", so], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.hex8_pressure_host.argtypes = [p, ctypes.c_int, ctypes.c_double, p]
    L.quad4_flux_host.argtypes = [p, ctypes.c_int, ctypes.c_double, ctypes.c_double, p]
    return L


@pytest.mark.parametrize("side", range(6))
def test_device_pressure_source_matches_the_oracle(side):
    L = _host()
    X = np.ascontiguousarray(brick(0.2, seed=10 + side).reshape(24))
    f = np.zeros(24)
    L.hex8_pressure_host(X, side, -2.5, f)
    ref = O.hex8_pressure(X, side, -2.5).reshape(3, 8).T.reshape(24)  # node-major
    assert np.abs(f - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("side", range(4))
def test_device_flux_source_matches_the_oracle(side):
    L = _host()
    X = np.ascontiguousarray(np.array([[0.0, 0.0], [2.0, 0.2], [2.3, 1.4], [-0.1, 1.0]]).reshape(8))
    f = np.zeros(4)
    L.quad4_flux_host(X, side, 5.0, 0.3, f)
    assert np.abs(f - O.quad4_heat_flux(X, side, 5.0, 0.3)).max() <= 1e-14
