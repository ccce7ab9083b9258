"""CPU-only checks of the C ABI library: it loads, exports every declared
symbol, and its host-side helpers agree with the oracle's mesh numbering."""
import ctypes
import os
import re

import numpy as np

import mastgpu as M
import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(REPO, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(mg_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = M.lib()
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_status_strings():
    L = M.lib()
    assert L.mg_version() == 1
    assert L.mg_status_string(M.MG_ENOCONV) == b"not converged"
    assert L.mg_status_string(12345) == b"unknown status"


def test_structured_grid_numbering_matches_oracle():
    c1, e1 = M.grid_hex8(4, 3, 2)
    c2, e2 = O.grid_hex8(4, 3, 2)
    assert np.array_equal(e1, e2) and np.allclose(c1, c2)
    q1, f1 = M.grid_quad4(5, 4)
    q2, f2 = O.grid_quad4(5, 4)
    assert np.array_equal(f1, f2) and np.allclose(q1, q2)


def test_problem_create_without_gpu_fails_cleanly():
    """With no CUDA device the library must report an error status, not crash."""
    import torch
    if torch.cuda.is_available():
        return
    coords, conn = M.grid_hex8(2, 1, 1)
    try:
        p = M.Problem(M.PHYS_HEX8, coords, conn, M.SIMP_MATERIAL)
    except M.MastGpuError as e:
        assert e.status in (M.MG_ECUDA, M.MG_ENOMEM)
    else:  # pragma: no cover - only on a GPU host
        p.close()


def test_batch_create_validates_before_touching_the_gpu():
    """Malformed designs are rejected with MG_EINVAL before any CUDA call; a
    well-formed batch on a host without a GPU reports MG_ECUDA."""
    import torch
    rho = np.full(8 * 4 * 4, 0.5)
    bad = [
        dict(nx=8, ny=4, nz=4, rho=np.full(128, 1.5), spans=[(0, 4)]),  # density > 1
        dict(nx=8, ny=4, nz=4, rho=rho, spans=[(3, 1)]),                # inverted span
        dict(nx=8, ny=4, nz=4, rho=rho, spans=[(0, 5)]),                # span beyond the edge
        dict(nx=0, ny=4, nz=4, rho=rho, spans=[(0, 4)]),                # empty grid
        dict(nx=8, ny=4, nz=4, rho=rho, spans=[]),                      # no load case
    ]
    for d in bad:
        try:
            M.Batch([d])
        except M.MastGpuError as e:
            assert e.status == M.MG_EINVAL, (d, e)
        else:  # pragma: no cover
            raise AssertionError("accepted %r" % (d,))
    if torch.cuda.is_available():
        return
    try:
        M.Batch([dict(nx=8, ny=4, nz=4, rho=rho, spans=[(0, 4)])])
    except M.MastGpuError as e:
        assert e.status in (M.MG_ECUDA, M.MG_ENOMEM)


def test_batch_designs_generator_is_seeded_and_in_range():
    a = M.batch_designs(12, seed=3)
    b = M.batch_designs(12, seed=3)
    for x, y in zip(a, b):
        assert (x["nx"], x["ny"], x["nz"]) == (y["nx"], y["ny"], y["nz"])
        assert np.array_equal(x["rho"], y["rho"]) and x["spans"] == y["spans"]
        assert (x["nx"], x["ny"], x["nz"]) in M.BATCH_SIZES
        assert 1 <= len(x["spans"]) <= 4
        assert all(0 <= j0 <= j1 <= x["ny"] for j0, j1 in x["spans"])
        assert x["rho"].min() >= 0.01 and x["rho"].max() <= 1.0


def test_output_entry_points_reject_missing_handles_without_a_gpu():
    """The adjoint, KS stress, sensitivity-solve, element and assembly-launch entry points
    check their arguments on
    the host first: a missing handle or vector is MG_EINVAL with no CUDA call."""
    L = M.lib()
    x = np.zeros(3)
    q, v = ctypes.c_double(), ctypes.c_double()
    assert L.mg_ks_stress(None, None, 8.0, 1.0, 0.5, ctypes.byref(q), ctypes.byref(v), None) == M.MG_EINVAL
    assert L.mg_adjoint_solve(None, M._p(x), M._p(x), None, M._p(x)) == M.MG_EINVAL
    assert L.mg_debug_launch_assembly(None, None, 1) == M.MG_EINVAL
    assert L.mg_compliance(None, None, None, None) == M.MG_EINVAL
    assert L.mg_sensitivity_solve(None, M._p(x), 0, 0, None, M._p(x)) == M.MG_EINVAL
    assert L.mg_output_derivative(None, 0, None, M._p(x)) == M.MG_EINVAL
    assert L.mg_element_calculations(None, 0, M._p(x), None, M._p(x)) == M.MG_EINVAL
    assert L.mg_element_sensitivity(None, 0, M._p(x), 0, 0, M._p(x)) == M.MG_EINVAL
    assert b"invalid argument" in L.mg_last_error()


def test_nonlinear_physics_value_is_the_header_enum():
    txt = open(os.path.join(REPO, "include", "mastgpu.h")).read()
    m = re.search(r"MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR\s*=\s*(\d+)", txt)
    assert m and int(m.group(1)) == M.PHYS_HEX8_NONLINEAR


def test_synthetic_request_regeneration_is_deterministic():
    """mg_server_synthetic_request is host code: it regenerates a request of the seeded
    synthetic stream (chain, grid, spans, densities) without a GPU."""
    d = M.synthetic_desc(50, 300.0, n_chains=5, sizes=((8, 4, 4), (16, 8, 8)), big_fraction=0.0,
                         max_cases=3, seed=9)
    by_chain = {}
    for i in range(50):
        a = M.synthetic_request(d, i)
        b = M.synthetic_request(d, i)
        assert a["chain"] == b["chain"] and a["spans"] == b["spans"]
        assert np.array_equal(a["rho"], b["rho"])
        nx, ny, nz = a["grid"]
        assert (nx, ny, nz) in ((8, 4, 4), (16, 8, 8)) and 1 <= len(a["spans"]) <= 3
        assert all(0 <= j0 <= j1 <= ny for j0, j1 in a["spans"])
        assert a["rho"].shape == (nx * ny * nz,)
        assert a["rho"].min() >= 0.01 - 1e-7 and a["rho"].max() <= 1.0
        by_chain.setdefault(a["chain"], []).append(a["rho"])
    # consecutive requests of a chain differ by the N(0, 0.02) step, clipped
    for seq in by_chain.values():
        for x, y in zip(seq, seq[1:]):
            dlt = np.abs(x - y)
            assert 0.0 < dlt.max() < 0.2 and 0.005 < dlt.mean() < 0.03
    bad = M.synthetic_desc(50, 300.0, n_chains=5)
    info = np.zeros(5, dtype=np.int32)
    assert M.lib().mg_server_synthetic_request(ctypes.byref(bad), 50, M._p(info), None, None) == M.MG_EINVAL
