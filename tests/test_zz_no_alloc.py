"""Allocation-free PCG entry point (mg_pcg_csr_static).

Some callers cannot call cudaMalloc: code that must not allocate after start-up
(a request loop held to a fixed device-memory budget) or a host application
whose own pool owns all device memory.  mg_pcg_csr_static serves them: they
pass their device buffers and the library keeps its scratch in one static
device array instead of allocating.  This test solves the 24x12x12 cantilever
system (12,675 dofs) through the C ABI twice in a row and checks each solution
against the existing entry point (mg_solve, plain FP64 Jacobi-PCG) within the
plain-form tolerance (1e-10 relative).  It lives in its own file, collected
last, and passes alone in a fresh process or after the other tests.
"""
import ctypes

import numpy as np
import pytest

import mastgpu as M

pytestmark = pytest.mark.gpu

RTOL_SOL = 1e-10


def _bind():
    L = M.lib()
    f = L.mg_pcg_csr_static
    f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int32,
                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    return f


def test_static_pcg_matches_mg_solve_twice():
    import torch
    nx, ny, nz = 24, 12, 12
    with M.simp_cantilever(nx, ny, nz) as p:
        p.set_design(np.full(nx * ny * nz, 0.5))
        u_ref, rep = p.solve(M.default_opts(rtol=1e-12))
        rowptr, cols, vals = p.get_csr()
        F = -p.residual_and_jacobian(np.zeros(p.n_dofs), want_J=False)  # R(0) = -F
    assert rep.status == 0
    dev = torch.device("cuda", 0)
    d_rowptr = torch.from_numpy(rowptr).to(dev)
    d_cols = torch.from_numpy(cols).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    d_b = torch.from_numpy(F).to(dev)
    stream = torch.cuda.current_stream(dev)
    solve = _bind()
    for call in range(2):
        d_x = torch.zeros(p.n_dofs, dtype=torch.float64, device=dev)
        its, rr = ctypes.c_int32(), ctypes.c_double()
        torch.cuda.synchronize()
        rc = solve(p.n_dofs, d_rowptr.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(),
                   d_b.data_ptr(), d_x.data_ptr(), 1e-12, 100000, stream.cuda_stream,
                   ctypes.byref(its), ctypes.byref(rr))
        torch.cuda.synchronize()
        assert rc == M.MG_OK, (call, rc, M.lib().mg_last_error())
        x = d_x.cpu().numpy()
        err = np.abs(x - u_ref).max() / np.abs(u_ref).max()
        assert err < RTOL_SOL, (call, err)
        assert rr.value <= 1e-12 and abs(its.value - rep.krylov_iterations) <= 5


def test_static_pcg_rejects_sizes_beyond_the_limit():
    solve = _bind()
    its, rr = ctypes.c_int32(), ctypes.c_double()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = solve(131072 + 1, dummy, dummy, dummy, dummy, dummy, 1e-8, 10, None,
               ctypes.byref(its), ctypes.byref(rr))
    assert rc == M.MG_EINVAL
    assert b"exceeds the static scratch limit" in M.lib().mg_last_error()
