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
