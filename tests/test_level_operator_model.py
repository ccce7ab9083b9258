"""CPU model of the factored multigrid level operator's sums (csrc/matfree.cu,
mf_fac_kernel): every element's corner results from the factored stiffness
(hex8_factored.cuh), then per node the fixed order the kernel uses -- along x
(left element's dx = 1 corner + right element's dx = 0 corner, a warp shuffle),
along y (lower element row + upper element row), along z (top corners of the
element plane below, carried in registers, + bottom corners of the plane above).
The order depends only on the node's eight elements, not on the tile a node falls
in, so the operator is deterministic and tiling-independent by construction; this
checks that the corner and bit conventions reproduce the assembled operator
sum_e E_e P_e^T K0 P_e u of the oracle's element routine (StructuralElement3D,
src/elasticity/solid_element_3d.cpp:135-423)."""
import os
import re

import numpy as np
import pytest

import oracle as O

HDR = os.path.join(os.path.dirname(__file__), "..", "mast-multiphysics_gb300", "csrc", "hex8_factored.cuh")


def terms():
    src = open(HDR).read()
    body = src[src.index("kFacTerms[kFacN][4] = {"):]
    body = body[:body.index("};")]
    return [tuple(int(v) for v in t) for t in re.findall(r"\{(\d), (\d), (\d), (\d)\}", body)]


def lex_to_node(b):
    bx, by, bz = b & 1, (b >> 1) & 1, (b >> 2) & 1
    return 4 * bz + ((2 if bx else 3) if by else (1 if bx else 0))


def unit_cube_K(nu=0.3):
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float)
    out = O.hex8_internal(X, 1.0, nu)
    return np.asarray(out[1] if isinstance(out, tuple) else out)  # dof c * 8 + a


def khat_values(K):
    A = [lex_to_node(b) for b in range(8)]
    h = np.array([[np.prod([((1 if (b >> t) & 1 else -1) if (m >> t) & 1 else 1) for t in range(3)])
                   for b in range(8)] for m in range(8)], dtype=float)
    kh = np.zeros((3, 8, 3, 8))
    for c in range(3):
        for d in range(3):
            kh[c, :, d, :] = h @ K[np.ix_([c * 8 + a for a in A], [d * 8 + a for a in A])] @ h.T / 64.0
    return [kh[c, m, d, mm] for (c, m, d, mm) in terms()]


def butterflies(v, forward):
    """8-point transform over the last axis (lexicographic corners / modes), in place order."""
    v = v.copy()
    for t in (1, 2, 4):
        for b in range(8):
            if not b & t:
                lo, hi = v[..., b].copy(), v[..., b | t].copy()
                if forward:
                    v[..., b], v[..., b | t] = lo + hi, hi - lo
                else:
                    v[..., b], v[..., b | t] = lo - hi, lo + hi
    return v


def level_operator(u, E, kv, tm):
    """u: (NZ, NY, NX, 3) nodes; E: (nz, ny, nx) elements -> (NZ, NY, NX, 3)."""
    nz, ny, nx = E.shape
    # corner values of every element, lexicographic corner b = bx + 2 by + 4 bz
    v = np.zeros((nz, ny, nx, 3, 8))
    for b in range(8):
        bx, by, bz = b & 1, (b >> 1) & 1, b >> 2
        v[..., b] = u[bz:bz + nz, by:by + ny, bx:bx + nx, :]
    vh = butterflies(v, True)
    yh = np.zeros_like(vh)
    for k, (c, m, d, mm) in enumerate(tm):
        yh[..., c, m] += kv[k] * vh[..., d, mm]
    yh *= E[..., None, None]
    yh[..., 0] = 0.0
    Y = butterflies(yh, False)  # (nz, ny, nx, 3, 8): e * K0 u_e at the corners
    pad = np.zeros((nz + 2, ny + 2, nx + 2, 3, 8))
    pad[1:-1, 1:-1, 1:-1] = Y  # element (ez, ey, ex) at pad[ez + 1, ey + 1, ex + 1]
    NZ, NY, NX = nz + 1, ny + 1, nx + 1
    k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")

    def corner(di, dj, dk, b):  # element (i - di, j - dj, k - dk), corner b
        return pad[k - dk + 1, j - dj + 1, i - di + 1, :, b]

    def xsum(dj, dk, by, bz):  # left element (dx = 1 corner) + right element (dx = 0 corner)
        return corner(1, dj, dk, 1 + 2 * by + 4 * bz) + corner(0, dj, dk, 2 * by + 4 * bz)

    def plane(dk, bz):  # lower element row (by = 1) + upper element row (by = 0)
        return xsum(1, dk, 1, bz) + xsum(0, dk, 0, bz)

    return plane(1, 1) + plane(0, 0)  # plane below (top corners) + plane above (bottom corners)


@pytest.mark.parametrize("shape", [(5, 4, 3), (40, 9, 7)])
def test_factored_sums_match_assembled_operator(shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(0)
    K = unit_cube_K()
    tm = terms()
    kv = khat_values(K)
    E = rng.uniform(0.01, 1.0, (nz, ny, nx))
    u = rng.normal(size=(nz + 1, ny + 1, nx + 1, 3))
    y = level_operator(u, E, kv, tm)
    # the same operator from the oracle's element matrix, element by element
    ref = np.zeros_like(u)
    A = [lex_to_node(b) for b in range(8)]
    for ez in range(nz):
        for ey in range(ny):
            for ex in range(nx):
                ue = np.zeros(24)
                for b in range(8):
                    bx, by, bz = b & 1, (b >> 1) & 1, b >> 2
                    for c in range(3):
                        ue[c * 8 + A[b]] = u[ez + bz, ey + by, ex + bx, c]
                fe = E[ez, ey, ex] * (K @ ue)
                for b in range(8):
                    bx, by, bz = b & 1, (b >> 1) & 1, b >> 2
                    for c in range(3):
                        ref[ez + bz, ey + by, ex + bx, c] += fe[c * 8 + A[b]]
    assert np.abs(y - ref).max() <= 1e-13 * np.abs(ref).max()
