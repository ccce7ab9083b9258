"""Nastran bulk data input (mg_bdf_*), the reader behind MAST::NastranIO::read
(src/mesh/nastran_io.cpp:221-339, read_nodes :105-125, read_elements :128-198,
read_node_boundaries :201-218).  A cantilever grid written as GRID / CHEXA /
SPC1 / FORCE cards in the three bulk data formats reads back as the structured
mesh of mastgpu.grid_hex8 (libMesh node order), with its clamp and tip load; the
GPU test solves the read mesh through the unstructured (coloured) assembly and
compares with the oracle."""
import numpy as np
import pytest

import mastgpu as M
import oracle as O


def small(*fields):
    """one small-field line: 8-column fields"""
    return "".join("%-8s" % str(f) for f in fields)


def large(*fields):
    return "%-8s" % str(fields[0]) + "".join("%16s" % str(f) for f in fields[1:])


def cantilever_bdf(nx, ny, nz, fmt="small", id0=101):
    coords, conn = M.grid_hex8(nx, ny, nz)
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    lines = ["$ cantilever %dx%dx%d" % (nx, ny, nz), "SOL 101", "CEND", "BEGIN BULK"]
    for i, (x, y, z) in enumerate(coords):
        gid = id0 + i
        if fmt == "small":
            lines.append(small("GRID", gid, "", "%.4f" % x, "%.4f" % y, "%.4f" % z))
        elif fmt == "large":
            lines.append(large("GRID*", gid, "", "%.8e" % x, "%.8e" % y))
            lines.append(large("*", "%.8e" % z))
        else:
            lines.append("GRID,%d,,%r,%r,%r" % (gid, float(x), float(y), float(z)))
    for e, nodes in enumerate(conn):
        g = [id0 + int(n) for n in nodes]
        if fmt == "free":
            lines.append("CHEXA,%d,1,%s" % (e + 1, ",".join(map(str, g[:6]))))
            lines.append(",%d,%d" % (g[6], g[7]))
        else:
            lines.append(small("CHEXA", e + 1, 1, *g[:6], "+E%d" % e))
            lines.append(small("+E%d" % e, *g[6:]))
    clamp = [id0 + NX * (j + NY * k) for k in range(NZ) for j in range(NY)]
    for a in range(0, len(clamp), 6):
        lines.append(small("SPC1", 1, 123, *clamp[a:a + 6]))
    tip = [id0 + nx + NX * j for j in range(NY)]
    for g in tip:
        lines.append(small("FORCE", 2, g, 0, "%.6g" % (1.0 / NY), 0.0, 0.0, -1.0))
    lines.append("ENDDATA")
    return "\n".join(lines) + "\n", coords, conn


@pytest.mark.parametrize("fmt", ["small", "large", "free"])
def test_cantilever_reads_back(fmt):
    nx, ny, nz = 4, 3, 2
    text, coords, conn = cantilever_bdf(nx, ny, nz, fmt)
    m = M.read_bdf(text=text)
    assert np.allclose(m["coords"], coords, atol=1e-4)
    assert np.array_equal(m["conn"], conn)
    assert np.array_equal(m["grid_ids"], 101 + np.arange(len(coords)))
    assert np.array_equal(m["elem_ids"], 1 + np.arange(len(conn)))
    assert np.array_equal(m["fixed_dofs"], np.sort(_fixed(nx, ny, nz)))
    NX = nx + 1
    tip = np.array([nx + NX * j for j in range(ny + 1)])
    assert np.array_equal(m["load_dofs"], 3 * tip + 2)
    assert np.allclose(m["load_values"], -1.0 / (ny + 1), rtol=1e-6)


def _fixed(nx, ny, nz):
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    k, j = np.meshgrid(np.arange(NZ), np.arange(NY), indexing="ij")
    clamp = (NX * (j + NY * k)).reshape(-1)
    return (clamp[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)


def test_nastran_reals_thru_and_quads():
    text = "\n".join([
        small("GRID", 7, "", "1.5-1", "-2.+1", ".25D0"),
        small("GRID", 3, "", "0.", "0.", "0."),
        small("GRID", 5, "", "1.0E0", "0.", "0."),
        small("GRID", 9, "", "1.", "1.", "0."),
        small("CQUAD4", 20, 4, 3, 5, 9, 7),
        small("SPC1", 1, 12, 3, "THRU", 5),
        small("SPC", 1, 9, 2, 0.0),
    ]) + "\n"
    m = M.read_bdf(text=text, dpn=2)
    # ascending GRID ids 3, 5, 7, 9 are nodes 0..3
    assert np.allclose(m["coords"][2], [0.15, -20.0, 0.25])
    assert np.array_equal(m["conn"], [[0, 1, 3, 2]]) and m["pids"][0] == 4
    # THRU 3..5 constrains GRIDs 3 and 5 (the absent 4 is skipped); a listed
    # undefined GRID is an error
    assert np.array_equal(m["fixed_dofs"], [0, 1, 2, 3, 7])
    with pytest.raises(RuntimeError):
        M.read_bdf(text=text + small("SPC1", 1, 1, 3, 4) + "\n", dpn=2)


@pytest.mark.parametrize("bad", [
    small("CHEXA", 1, 1, 1, 2, 3, 4, 5, 6) + "\n" + small("+", 7, 99) + "\n",  # undefined GRID 99
    small("SPC", 1, 1, 1, 0.5) + "\n",                                        # non-zero enforced value
    small("GRID", 50, 2, 0.0, 0.0, 0.0) + "\n",                               # a local coordinate system
])
def test_malformed_cards_are_rejected(bad):
    grids = "".join(small("GRID", i, "", float(i), 0.0, 0.0) + "\n" for i in range(1, 9))
    with pytest.raises(RuntimeError):
        M.read_bdf(text=grids + small("CHEXA", 2, 1, 1, 2, 3, 4, 5, 6) + "\n" + small("+", 7, 8) + "\n" + bad)


@pytest.mark.gpu
def test_bdf_cantilever_solves_like_the_oracle():
    nx, ny, nz = 8, 4, 4
    text, _, _ = cantilever_bdf(nx, ny, nz, "small", id0=1001)
    m = M.read_bdf(text=text)
    rho = np.random.default_rng(5).uniform(0.2, 1.0, nx * ny * nz)
    with M.Problem(M.PHYS_HEX8, m["coords"], m["conn"], M.SIMP_MATERIAL, fixed_dofs=m["fixed_dofs"],
                   load_dofs=m["load_dofs"], load_values=m["load_values"]) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-12))
        c, dc = p.compliance()
    u_ref, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-13), rho)
    assert rep.status == 0
    assert np.abs(u - u_ref).max() <= 1e-9 * np.abs(u_ref).max()
    assert abs(c - r.compliance) <= 1e-10 * abs(r.compliance)
    assert np.abs(dc - dc_ref).max() <= 1e-9 * np.abs(dc_ref).max()
