"""The factored element stiffness used by the CUDA-core operators (FP64
refinement residual, FP32 multigrid level operator): in the per-axis
sum/difference basis of the 2x2x2 corners, the HEX8 stiffness of a box element
(StructuralElement3D, src/elasticity/structural_element_3d.cpp:135-423, 2x2x2
Gauss) has nonzeros only at the 45 (component, mode) pairs listed in
csrc/hex8_factored.cuh.  Checked against the oracle's element routine for
several aspect ratios and Poisson ratios, and the factored product against the
dense one."""
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
    """lexicographic corner b = bx + 2 by + 4 bz -> element node a (libMesh HEX8)"""
    bx, by, bz = b & 1, (b >> 1) & 1, (b >> 2) & 1
    return 4 * bz + ((2 if bx else 3) if by else (1 if bx else 0))


def H():
    h = np.zeros((8, 8))
    for m in range(8):
        for b in range(8):
            h[m, b] = np.prod([((1 if (b >> t) & 1 else -1) if (m >> t) & 1 else 1) for t in range(3)])
    return h


def box_stiffness(hx, hy, hz, nu):
    X = np.array([[0, 0, 0], [hx, 0, 0], [hx, hy, 0], [0, hy, 0],
                  [0, 0, hz], [hx, 0, hz], [hx, hy, hz], [0, hy, hz]], dtype=float)
    out = O.hex8_internal(X, 1.0, nu)
    return np.asarray(out[1] if isinstance(out, tuple) else out)  # dof c * 8 + a


def khat(K):
    A = [lex_to_node(b) for b in range(8)]
    h = H()
    kh = np.zeros((3, 8, 3, 8))
    for c in range(3):
        for d in range(3):
            blk = K[np.ix_([c * 8 + a for a in A], [d * 8 + a for a in A])]
            kh[c, :, d, :] = h @ blk @ h.T / 64.0
    return kh


def test_table_has_45_distinct_terms():
    t = terms()
    assert len(t) == 45 and len(set(t)) == 45
    assert all(m > 0 and mm > 0 for (_, m, _, mm) in t)  # rigid translations (mode 0) drop out


@pytest.mark.parametrize("box", [(1, 1, 1, 0.3), (1, 2, 0.5, 0.3), (0.7, 1.3, 1.1, 0.45), (1, 1, 1, 0.0)])
def test_stiffness_vanishes_outside_the_table(box):
    kh = khat(box_stiffness(*box))
    mask = np.zeros(kh.shape, dtype=bool)
    for (c, m, d, mm) in terms():
        mask[c, m, d, mm] = True
    assert np.abs(kh[~mask]).max() <= 1e-13 * np.abs(kh).max()


def test_factored_product_matches_dense():
    K = box_stiffness(1.0, 2.0, 0.5, 0.3)
    kh = khat(K)
    h = H()
    A = [lex_to_node(b) for b in range(8)]
    rng = np.random.default_rng(0)
    for _ in range(5):
        u = rng.normal(size=24)  # c * 8 + a
        v = np.array([[u[c * 8 + A[b]] for b in range(8)] for c in range(3)])
        vh = v @ h.T  # forward butterflies: mode m = sum_b H[m, b] v[b]
        yh = np.zeros((3, 8))
        for (c, m, d, mm) in terms():
            yh[c, m] += kh[c, m, d, mm] * vh[d, mm]
        y_lex = yh @ h  # back: corner b = sum_m H[m, b] yh[m]
        y = np.zeros(24)
        for c in range(3):
            for b in range(8):
                y[c * 8 + A[b]] = y_lex[c, b]
        assert np.abs(y - K @ u).max() <= 1e-14 * np.abs(K @ u).max()
