"""ExodusII files (MAST writes its solutions through libMesh's ExodusII_IO,
examples/structural/example_7/example_7.cpp:256-281).

The writer's files are read back by an independent netCDF classic reader
(scipy.io.netcdf_file) and checked against the ExodusII data model: dimensions,
coordinates, 1-based connectivity with its elem_type, the variable name tables
and values of the time step.  The reader takes files that scipy writes itself
(CDF-1 and CDF-2, two element blocks), and a mesh read from such a file solves
like the oracle's grid."""
import os

import numpy as np
import pytest

import mastgpu as M
import oracle as O

netcdf_file = pytest.importorskip("scipy.io").netcdf_file


def names(var):
    return ["".join(c.decode() for c in row if c != b"").strip("\x00") for row in var[:]]


def test_written_file_reads_back_with_an_independent_netcdf_reader(tmp_path):
    coords, conn = M.grid_hex8(3, 2, 2)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((coords.shape[0], 3))
    rho = rng.uniform(0.1, 1.0, conn.shape[0])
    path = str(tmp_path / "cantilever.exo")
    M.write_exodus(path, coords, conn, nodal={"disp_x": u[:, 0], "disp_y": u[:, 1], "disp_z": u[:, 2]},
                   elem={"rho": rho}, title="SIMP cantilever", time=1.5)
    with netcdf_file(path, "r", mmap=False) as f:
        assert f.version_byte == 2
        d = f.dimensions
        assert d["num_dim"] == 3 and d["num_nodes"] == coords.shape[0] and d["num_elem"] == conn.shape[0]
        assert d["num_el_blk"] == 1 and d["num_nod_per_el1"] == 8 and d["time_step"] is None
        for k, ax in enumerate(("coordx", "coordy", "coordz")):
            assert np.array_equal(f.variables[ax][:], coords[:, k])
        c = f.variables["connect1"]
        assert np.array_equal(c[:], conn + 1)
        assert c.elem_type == b"HEX8"
        assert names(f.variables["name_nod_var"]) == ["disp_x", "disp_y", "disp_z"]
        assert names(f.variables["name_elem_var"]) == ["rho"]
        assert np.array_equal(f.variables["time_whole"][:], [1.5])
        for k in range(3):
            assert np.array_equal(f.variables["vals_nod_var%d" % (k + 1)][0], u[:, k])
        assert np.array_equal(f.variables["vals_elem_var1eb1"][0], rho)
        assert f.title == b"SIMP cantilever"
    c2, k2 = M.read_exodus(path)
    assert np.array_equal(c2, coords) and np.array_equal(k2, conn)


@pytest.mark.parametrize("version", [1, 2])
def test_reader_takes_classic_files_with_several_blocks(tmp_path, version):
    coords, conn = M.grid_hex8(4, 2, 1)
    half = conn.shape[0] // 2
    path = str(tmp_path / ("blocks_v%d.exo" % version))
    with netcdf_file(path, "w", version=version) as f:
        f.createDimension("num_dim", 3)
        f.createDimension("num_nodes", coords.shape[0])
        f.createDimension("num_elem", conn.shape[0])
        f.createDimension("num_el_blk", 2)
        f.createDimension("num_el_in_blk1", half)
        f.createDimension("num_el_in_blk2", conn.shape[0] - half)
        f.createDimension("num_nod_per_el1", 8)
        f.createDimension("num_nod_per_el2", 8)
        # the packed coordinate form: coord[num_dim][num_nodes]
        v = f.createVariable("coord", "d", ("num_dim", "num_nodes"))
        v[:] = coords.T
        for b, (lo, hi) in enumerate(((0, half), (half, conn.shape[0]))):
            v = f.createVariable("connect%d" % (b + 1), "i", ("num_el_in_blk%d" % (b + 1), "num_nod_per_el%d" % (b + 1)))
            v[:] = conn[lo:hi] + 1
            v.elem_type = "HEX8"
    c2, k2 = M.read_exodus(path)
    assert np.array_equal(c2, coords) and np.array_equal(k2, conn)


def test_not_a_classic_file_is_rejected(tmp_path):
    bad = tmp_path / "bad.exo"
    bad.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))  # a netCDF-4 / HDF5 signature
    with pytest.raises(M.MastGpuError) as e:
        M.read_exodus(str(bad))
    assert e.value.status == M.MG_EINVAL
    with pytest.raises(M.MastGpuError):
        M.write_exodus(str(tmp_path / "x.exo"), np.zeros((8, 3)), np.full((1, 8), 9, np.int32))  # node 9 of 8


def _hex_file(path, conn_values, conn_type="i", record=False):
    coords, _ = M.grid_hex8(1, 1, 1)
    with netcdf_file(path, "w", version=2) as f:
        f.createDimension("time_step", None)
        f.createDimension("num_dim", 3)
        f.createDimension("num_nodes", coords.shape[0])
        f.createDimension("num_elem", 1)
        f.createDimension("num_el_blk", 1)
        f.createDimension("num_el_in_blk1", 1)
        f.createDimension("num_nod_per_el1", 8)
        for k, ax in enumerate(("coordx", "coordy", "coordz")):
            f.createVariable(ax, "d", ("num_nodes",))[:] = coords[:, k]
        dims = ("time_step", "num_nod_per_el1") if record else ("num_el_in_blk1", "num_nod_per_el1")
        v = f.createVariable("connect1", conn_type, dims)
        v[:] = np.asarray(conn_values).reshape(1, 8)
        v.elem_type = "HEX8"


def test_malformed_files_are_rejected(tmp_path):
    """Headers and tables that do not describe the data are errors, never reads or
    writes outside the file or the caller's arrays: a truncated file, a connectivity
    stored as a record variable, node numbers that are not integers in 1..num_nodes."""
    good = str(tmp_path / "good.exo")
    _hex_file(good, np.arange(1, 9))
    c, k = M.read_exodus(good)
    assert c.shape == (8, 3) and np.array_equal(k[0], np.arange(8))
    raw = open(good, "rb").read()
    for cut in (len(raw) - 4, len(raw) // 2, 12):
        bad = tmp_path / ("cut%d.exo" % cut)
        bad.write_bytes(raw[:cut])
        with pytest.raises(M.MastGpuError) as e:
            M.read_exodus(str(bad))
        assert e.value.status == M.MG_EINVAL
    cases = {"record.exo": dict(conn_values=np.arange(1, 9), record=True),
             "nan.exo": dict(conn_values=[1, 2, 3, 4, 5, 6, 7, np.nan], conn_type="d"),
             "frac.exo": dict(conn_values=[1, 2, 3, 4, 5, 6, 7, 7.5], conn_type="d"),
             "zero.exo": dict(conn_values=[0, 2, 3, 4, 5, 6, 7, 8]),
             "high.exo": dict(conn_values=[1, 2, 3, 4, 5, 6, 7, 9])}
    for name, kw in cases.items():
        path = str(tmp_path / name)
        _hex_file(path, **kw)
        with pytest.raises(M.MastGpuError) as e:
            M.read_exodus(path)
        assert e.value.status == M.MG_EINVAL, name


def test_writer_rejects_unnamed_variables(tmp_path):
    """A null entry in a name table is an argument error of the C ABI, not a crash."""
    import ctypes
    coords, conn = M.grid_hex8(1, 1, 1)
    coords = np.ascontiguousarray(coords)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    vals = np.zeros(2 * coords.shape[0])  # two nodal variables, kept alive over the call
    names = (ctypes.c_char_p * 2)(b"a", None)
    rc = M.lib().mg_exodus_write(os.fsencode(str(tmp_path / "x.exo")), None, 3, 8, coords.shape[0],
                                 coords.ctypes.data, conn.shape[0], conn.ctypes.data, 2, names,
                                 vals.ctypes.data, 0, None, None, 0.0)
    assert rc == M.MG_EINVAL
    assert not (tmp_path / "x.exo").exists()


@pytest.mark.gpu
def test_exodus_mesh_solves_like_the_oracle(tmp_path):
    """A cantilever mesh written to ExodusII and read back, clamped and loaded as
    the oracle's grid, solves to the oracle's answer; the solution and densities
    go back out as nodal and element variables."""
    nx, ny, nz = 8, 4, 4
    coords, conn = M.grid_hex8(nx, ny, nz)
    path = str(tmp_path / "mesh.exo")
    M.write_exodus(path, coords, conn)
    c2, k2 = M.read_exodus(path)
    rho = np.random.default_rng(6).uniform(0.2, 1.0, nx * ny * nz)
    ref = M.simp_cantilever(nx, ny, nz)
    with M.Problem(M.PHYS_HEX8, c2, k2, M.SIMP_MATERIAL, fixed_dofs=ref.fixed_dofs, load_dofs=ref.load_dofs,
                   load_values=ref.load_values) as p:
        p.set_design(rho)
        u, rep = p.solve(M.default_opts(rtol=1e-12))
        c, dc = p.compliance()
    ref.close()
    u_ref, dc_ref, r = O.simp_solve(O.simp_desc(nx, ny, nz, rtol=1e-13), rho)
    assert rep.status == 0
    assert np.abs(u - u_ref).max() <= 1e-9 * np.abs(u_ref).max()
    assert abs(c - r.compliance) <= 1e-10 * abs(r.compliance)
    out = str(tmp_path / "solution.exo")
    uu = u.reshape(-1, 3)
    M.write_exodus(out, c2, k2, nodal={"disp_x": uu[:, 0], "disp_y": uu[:, 1], "disp_z": uu[:, 2]},
                   elem={"rho": rho, "dc_drho": dc})
    with netcdf_file(out, "r", mmap=False) as f:
        assert np.array_equal(f.variables["vals_nod_var3"][0], uu[:, 2])
        assert np.array_equal(f.variables["vals_elem_var2eb1"][0], dc)
