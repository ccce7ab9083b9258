"""Python binding of libmastgpu.so (the C ABI in include/mastgpu.h).

The product is the CUDA/C++ library; this module builds it in-tree with nvcc
for sm_103a and exposes the ABI through ctypes for tests, the benchmark and
Python callers.  It contains no numerical fallback: every operation below calls
the library, and loading fails loudly when the library is missing.

Structured-mesh helpers reproduce the libMesh build_cube / build_square
numbering the reference's examples use (examples/structural/base/
bracket_3d_model.h:172-205 calls MeshTools::Generation::build_cube).
"""
import ctypes
import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libmastgpu.so")
INCLUDE = os.path.join(REPO, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def build(force=False, verbose=False):
    """Compile every CUDA translation unit for sm_103a and link libmastgpu.so."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_mtime):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (s, r.stdout, r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr)
        return o

    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(compile_one, jobs))
    if force or jobs or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB_PATH] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB_PATH


# --------------------------------------------------------------------------- ABI
MG_OK, MG_EINVAL, MG_ENOMEM, MG_ENOCONV, MG_EBREAKDOWN, MG_ENAN = 0, -1, -2, -3, -4, -5
MG_ETIMEDOUT, MG_ECUDA, MG_ENOTSUP, MG_EBUSY, MG_EBADELEM = -6, -7, -8, -9, -10
PHYS_HEX8, PHYS_MEMBRANE, PHYS_HEAT = 0, 1, 2
PHYS_HEX8_NONLINEAR = 3  # Green-Lagrange strain (MAST::NONLINEAR_STRAIN), Newton
PLAIN_FP64, MIXED_TF32, MIXED_BF16, MIXED_TF32X3, MIXED_BF16X3 = 0, 1, 2, 3, 4
KRYLOV_CG, KRYLOV_BICGSTAB = 0, 1
OUTPUT_COMPLIANCE, OUTPUT_MEAN_TEMPERATURE = 0, 1
PC_JACOBI, PC_MULTIGRID = 0, 1
SMOOTHER_FACTORED, SMOOTHER_TENSOR = 0, 1
OPERATOR_FACTORED_FP32 = 100  # mg_debug_matfree_apply / mg_debug_launch_apply: factored FP32 operator
PARAM_DENSITY, PARAM_K0, PARAM_ELEM_SCALE = 0, 1, 2

_vp = ctypes.c_void_p
_i32, _i64, _dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_double


class MeshDesc(ctypes.Structure):
    _fields_ = [("physics", _i32), ("reserved0", _i32), ("n_nodes", _i64), ("n_elems", _i64),
                ("coords", _vp), ("conn", _vp), ("grid_nx", _i32), ("grid_ny", _i32),
                ("grid_nz", _i32), ("reserved1", _i32)]


class MaterialDesc(ctypes.Structure):
    _fields_ = [("E0", _dbl), ("Emin", _dbl), ("nu", _dbl), ("penal", _dbl), ("thickness", _dbl),
                ("k0", _dbl), ("k_beta", _dbl)]


class BcDesc(ctypes.Structure):
    _fields_ = [("n_fixed", _i64), ("fixed_dofs", _vp), ("n_point_loads", _i64),
                ("load_dofs", _vp), ("load_values", _vp), ("n_conv", _i64), ("conv_elems", _vp),
                ("conv_sides", _vp), ("conv_h", _dbl), ("conv_Tinf", _dbl),
                ("source_elem", _vp)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("precision", _i32), ("krylov", _i32), ("max_iterations", _i32),
                ("max_newton", _i32), ("rtol", _dbl), ("newton_rtol", _dbl),
                ("consistent_jacobian", _i32), ("max_refinements", _i32), ("inner_rtol", _dbl),
                ("timeout_s", _dbl), ("warm_start", _i32), ("graph_chunk", _i32),
                ("preconditioner", _i32), ("smooth_degree", _i32), ("coarse_degree", _i32),
                ("vec_blocks_per_sm", _i32), ("smoother_operator", _i32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_cap_bytes", _i64), ("solve", SolveOpts), ("max_inflight", _i32),
                ("reserved", _i32)]


class BatchProblem(ctypes.Structure):
    _fields_ = [("nx", _i32), ("ny", _i32), ("nz", _i32), ("n_cases", _i32), ("rho", _vp),
                ("span", _vp), ("F", _vp), ("node_fix", _vp)]


class Request(ctypes.Structure):
    _fields_ = [("chain", _i32), ("nx", _i32), ("ny", _i32), ("nz", _i32), ("n_cases", _i32),
                ("reserved", _i32), ("rho", _vp), ("span", _vp), ("compliance_out", _vp),
                ("dc_out", _vp), ("arrival_s", _dbl), ("tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("chain", _i32), ("status", _i32),
                ("krylov_iterations", _i32), ("refinements", _i32), ("relres", _dbl),
                ("arrival_s", _dbl), ("admit_s", _dbl), ("done_s", _dbl)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", _i64), ("completed", _i64), ("failed", _i64), ("rebuilds", _i64),
                ("evictions", _i64), ("resident_bytes", _i64), ("peak_resident_bytes", _i64),
                ("resident_chains", _i32), ("inflight", _i32), ("peak_inflight", _i32),
                ("reserved", _i32), ("p50_s", _dbl), ("p99_s", _dbl), ("mean_s", _dbl),
                ("max_s", _dbl), ("solves_per_s", _dbl), ("dofs_per_s", _dbl)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_ if f[0] != "reserved"}


class SyntheticDesc(ctypes.Structure):
    _fields_ = [("n_requests", _i64), ("rate", _dbl), ("n_chains", _i32), ("n_sizes", _i32),
                ("sizes", _vp), ("big_fraction", _dbl), ("big_nx", _i32), ("big_ny", _i32),
                ("big_nz", _i32), ("max_cases", _i32), ("noise", _dbl), ("seed", ctypes.c_uint64)]


class SolveReport(ctypes.Structure):
    _fields_ = [("status", _i32), ("newton_iterations", _i32), ("krylov_iterations", _i32),
                ("refinements", _i32), ("relres", _dbl), ("residual_norm", _dbl),
                ("seconds", _dbl)]


_lib = None


def lib(autobuild=True):
    """Load libmastgpu.so (building it first if needed); raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if autobuild:
        build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libmastgpu.so is not built (%s)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    L.mg_version.restype = ctypes.c_int
    L.mg_status_string.restype = ctypes.c_char_p
    L.mg_status_string.argtypes = [ctypes.c_int]
    L.mg_last_error.restype = ctypes.c_char_p
    L.mg_device_info.argtypes = [ctypes.c_char_p, ctypes.c_int, _vp, _vp, _vp]
    L.mg_default_solve_opts.argtypes = [ctypes.POINTER(SolveOpts)]
    L.mg_default_solve_opts.restype = None
    L.mg_problem_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(MaterialDesc),
                                    ctypes.POINTER(BcDesc), ctypes.POINTER(_vp)]
    L.mg_problem_destroy.argtypes = [_vp]
    L.mg_problem_destroy.restype = None
    L.mg_problem_info.argtypes = [_vp, _vp, _vp, _vp]
    L.mg_problem_stream.argtypes = [_vp]
    L.mg_problem_stream.restype = _vp
    L.mg_set_design.argtypes = [_vp, _vp]
    L.mg_set_design_device.argtypes = [_vp, _vp]
    L.mg_set_design_nodal.argtypes = [_vp, _vp]
    L.mg_set_elem_scale.argtypes = [_vp, _vp]
    L.mg_residual_and_jacobian.argtypes = [_vp, _vp, _vp, ctypes.c_int]
    L.mg_get_csr.argtypes = [_vp, _vp, _vp, _vp]
    L.mg_element_matrices.argtypes = [_vp, _vp, _i64, _i64, _vp, _vp]
    L.mg_spmv.argtypes = [_vp, _vp, _vp]
    L.mg_solve.argtypes = [_vp, ctypes.POINTER(SolveOpts), _vp, ctypes.POINTER(SolveReport)]
    L.mg_get_solution.argtypes = [_vp, _vp]
    L.mg_solution_device.argtypes = [_vp]
    L.mg_solution_device.restype = _vp
    L.mg_sensitivity_assemble.argtypes = [_vp, _vp, _i32, _i64, _vp]
    L.mg_compliance.argtypes = [_vp, _vp, _vp, _vp]
    L.mg_adjoint_solve.argtypes = [_vp, _vp, _vp, ctypes.POINTER(SolveOpts), _vp]
    L.mg_ks_stress.argtypes = [_vp, _vp, _dbl, _dbl, _dbl, _vp, _vp, _vp]
    L.mg_set_side_loads.argtypes = [_vp, _i64, _vp, _vp, _vp]
    L.mg_mean_temperature.argtypes = [_vp, _vp, ctypes.POINTER(SolveOpts), _vp, _vp, _vp]
    L.mg_sensitivity_solve.argtypes = [_vp, _vp, _i32, _i64, ctypes.POINTER(SolveOpts), _vp]
    L.mg_output_derivative.argtypes = [_vp, _i32, _vp, _vp]
    L.mg_element_calculations.argtypes = [_vp, _i64, _vp, _vp, _vp]
    L.mg_element_sensitivity.argtypes = [_vp, _i64, _vp, _i32, _i64, _vp]
    L.mg_debug_matfree_apply.argtypes = [_vp, ctypes.c_int, _vp, _vp]
    L.mg_compliance_resident.argtypes = [_vp, _vp]
    L.mg_sensitivities_device.argtypes = [_vp]
    L.mg_sensitivities_device.restype = _vp
    L.mg_launch_count.restype = ctypes.c_longlong
    L.mg_debug_launch_apply.argtypes = [_vp, ctypes.c_int, ctypes.c_int]
    L.mg_debug_launch_assembly.argtypes = [_vp, _vp, ctypes.c_int]
    L.mg_debug_fail_alloc_after.argtypes = [ctypes.c_int]
    L.mg_debug_fail_alloc_after.restype = None
    L.mg_batch_create.argtypes = [ctypes.POINTER(BatchProblem), _i32, ctypes.POINTER(MaterialDesc),
                                  ctypes.POINTER(_vp)]
    L.mg_batch_destroy.argtypes = [_vp]
    L.mg_batch_destroy.restype = None
    L.mg_batch_info.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp]
    L.mg_batch_stream.argtypes = [_vp]
    L.mg_batch_stream.restype = _vp
    L.mg_batch_set_design.argtypes = [_vp, _i32, _vp]
    L.mg_batch_set_design_device.argtypes = [_vp, _i32, _vp]
    L.mg_batch_solve.argtypes = [_vp, ctypes.POINTER(SolveOpts), _vp]
    L.mg_batch_solve_subset.argtypes = [_vp, ctypes.POINTER(SolveOpts), _vp, _vp]
    L.mg_batch_results.argtypes = [_vp, _i32, _vp, _vp, _vp]
    L.mg_batch_autotune.argtypes = [_vp, ctypes.POINTER(SolveOpts), _i32, _vp]
    L.mg_filter_create_grid.argtypes = [_i32, _i32, _i32, _dbl, _dbl, _dbl, _dbl, _vp, ctypes.POINTER(_vp)]
    L.mg_filter_create_points.argtypes = [_i64, _i32, _vp, _dbl, _vp, ctypes.POINTER(_vp)]
    L.mg_filter_info.argtypes = [_vp, _vp, _vp]
    L.mg_filter_apply.argtypes = [_vp, _vp, _vp, _i32]
    L.mg_filter_apply_device.argtypes = [_vp, _vp, _vp, _i32, _vp]
    L.mg_filter_destroy.argtypes = [_vp]
    L.mg_filter_destroy.restype = None
    L.mg_bdf_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(_vp)]
    L.mg_exodus_write.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _i32, _i32, _i64, _vp, _i64, _vp, _i32,
                                  ctypes.POINTER(ctypes.c_char_p), _vp, _i32, ctypes.POINTER(ctypes.c_char_p),
                                  _vp, ctypes.c_double]
    L.mg_exodus_read_sizes.argtypes = [ctypes.c_char_p, ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                       ctypes.POINTER(_i64), ctypes.POINTER(_i64)]
    L.mg_exodus_read_mesh.argtypes = [ctypes.c_char_p, _vp, _vp]
    L.mg_bdf_parse.argtypes = [ctypes.c_char_p, _i64, ctypes.POINTER(_vp)]
    L.mg_bdf_sizes.argtypes = [_vp, _vp, _vp, _vp]
    L.mg_bdf_nodes.argtypes = [_vp, _vp, _vp]
    L.mg_bdf_elements.argtypes = [_vp, _vp, _vp, _vp]
    L.mg_bdf_constraints.argtypes = [_vp, _i32, _vp, _vp]
    L.mg_bdf_loads.argtypes = [_vp, _i32, _vp, _vp, _vp]
    L.mg_bdf_destroy.argtypes = [_vp]
    L.mg_bdf_destroy.restype = None
    L.mg_server_clock.restype = ctypes.c_double
    L.mg_server_create.argtypes = [ctypes.POINTER(MaterialDesc), ctypes.POINTER(ServerOpts),
                                   ctypes.POINTER(_vp)]
    L.mg_server_submit.argtypes = [_vp, ctypes.POINTER(Request)]
    L.mg_server_poll.argtypes = [_vp, _vp, _i32, _vp, ctypes.c_double]
    L.mg_server_drain.argtypes = [_vp, ctypes.c_double]
    L.mg_server_get_stats.argtypes = [_vp, ctypes.POINTER(ServerStats)]
    L.mg_server_destroy.argtypes = [_vp]
    L.mg_server_destroy.restype = None
    L.mg_server_run_synthetic.argtypes = [_vp, ctypes.POINTER(SyntheticDesc), _vp,
                                          ctypes.POINTER(ServerStats)]
    L.mg_server_synthetic_request.argtypes = [ctypes.POINTER(SyntheticDesc), _i64, _vp, _vp, _vp]
    _lib = L
    return L


class MastGpuError(RuntimeError):
    def __init__(self, status, where):
        L = lib(False)
        msg = L.mg_status_string(status).decode()
        detail = L.mg_last_error().decode()
        super().__init__("%s: %s (%d) %s" % (where, msg, status, detail))
        self.status = status


def check(status, where):
    if status != MG_OK:
        raise MastGpuError(status, where)


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def default_opts(**kw):
    """mg_default_solve_opts with the given fields replaced; the host wall-clock
    limit defaults to 600 s here (the C default is none)."""
    o = SolveOpts()
    lib().mg_default_solve_opts(ctypes.byref(o))
    o.timeout_s = 600.0
    for k, v in kw.items():
        setattr(o, k, v)
    return o


# ------------------------------------------------------------------ structured meshes
def grid_hex8(nx, ny, nz, lx=None, ly=None, lz=None):
    """Unit-spaced (by default) HEX8 grid in libMesh build_cube numbering."""
    lx = float(nx if lx is None else lx)
    ly = float(ny if ly is None else ly)
    lz = float(nz if lz is None else lz)
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([i * (lx / nx), j * (ly / ny), k * (lz / nz)], axis=-1).reshape(-1, 3)
    NX, NY = nx + 1, ny + 1
    ke, je, ie = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n0 = (ie + NX * (je + NY * ke)).reshape(-1)
    off = np.array([0, 1, 1 + NX, NX, NX * NY, 1 + NX * NY, 1 + NX + NX * NY, NX + NX * NY])
    conn = (n0[:, None] + off[None, :]).astype(np.int32)
    return np.ascontiguousarray(coords, dtype=np.float64), np.ascontiguousarray(conn)


def grid_quad4(nx, ny, lx=1.0, ly=1.0):
    j, i = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([i * (lx / nx), j * (ly / ny)], axis=-1).reshape(-1, 2)
    NX = nx + 1
    je, ie = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    n0 = (ie + NX * je).reshape(-1)
    conn = (n0[:, None] + np.array([0, 1, 1 + NX, NX])[None, :]).astype(np.int32)
    return np.ascontiguousarray(coords, dtype=np.float64), np.ascontiguousarray(conn)


# ------------------------------------------------------------------ problem handle
class Problem:
    """One mg_problem handle (mesh + design + device system on one stream)."""

    def __init__(self, physics, coords, conn, material, fixed_dofs=(), load_dofs=(),
                 load_values=(), conv_elems=(), conv_sides=(), conv_h=0.0, conv_Tinf=0.0,
                 source_elem=None, grid=(0, 0, 0)):
        L = lib()
        self._keep = []
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.physics = physics
        self.dpn = {PHYS_HEX8: 3, PHYS_HEX8_NONLINEAR: 3, PHYS_MEMBRANE: 2, PHYS_HEAT: 1}[physics]
        self.n_nodes = self.coords.shape[0]
        self.n_elems = self.conn.shape[0]
        self.n_dofs = self.n_nodes * self.dpn
        # the boundary conditions as given (to rebuild the same problem on another mesh)
        self.fixed_dofs = np.asarray(fixed_dofs, dtype=np.int64).copy()
        self.load_dofs = np.asarray(load_dofs, dtype=np.int64).copy()
        self.load_values = np.asarray(load_values, dtype=np.float64).copy()
        mesh = MeshDesc(physics, 0, self.n_nodes, self.n_elems, _p(self.coords), _p(self.conn),
                        grid[0], grid[1], grid[2], 0)
        mat = MaterialDesc(**material)
        fx = np.ascontiguousarray(fixed_dofs, dtype=np.int64)
        ld = np.ascontiguousarray(load_dofs, dtype=np.int64)
        lv = np.ascontiguousarray(load_values, dtype=np.float64)
        ce = np.ascontiguousarray(conv_elems, dtype=np.int32)
        cs = np.ascontiguousarray(conv_sides, dtype=np.int32)
        src = None if source_elem is None else np.ascontiguousarray(source_elem, dtype=np.float64)
        self._keep += [fx, ld, lv, ce, cs, src]
        bc = BcDesc(fx.shape[0], _p(fx), ld.shape[0], _p(ld), _p(lv), ce.shape[0], _p(ce), _p(cs),
                    conv_h, conv_Tinf, _p(src))
        h = ctypes.c_void_p()
        check(L.mg_problem_create(ctypes.byref(mesh), ctypes.byref(mat), ctypes.byref(bc),
                                  ctypes.byref(h)), "mg_problem_create")
        self.h = h
        n = ctypes.c_int64()
        nnz = ctypes.c_int64()
        nc = ctypes.c_int32()
        check(L.mg_problem_info(self.h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nc)),
              "mg_problem_info")
        self.nnz, self.n_colors = nnz.value, nc.value

    def close(self):
        if getattr(self, "h", None):
            lib().mg_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return lib().mg_problem_stream(self.h)

    def set_design(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        check(lib().mg_set_design(self.h, _p(rho)), "mg_set_design")
        self.nodal = False

    def set_design_device(self, ptr):
        check(lib().mg_set_design_device(self.h, ctypes.c_void_p(ptr)), "mg_set_design_device")
        self.nodal = False

    def set_design_nodal(self, rho_nodes):
        """Nodal density field (n_nodes values): the modulus per Gauss point from
        the trilinear field (mg_set_design_nodal); compliance() then returns
        dC/drho per node."""
        rho_nodes = np.ascontiguousarray(rho_nodes, dtype=np.float64)
        check(lib().mg_set_design_nodal(self.h, _p(rho_nodes)), "mg_set_design_nodal")
        self.nodal = True

    def set_elem_scale(self, s):
        s = np.ascontiguousarray(s, dtype=np.float64)
        check(lib().mg_set_elem_scale(self.h, _p(s)), "mg_set_elem_scale")

    def residual_and_jacobian(self, X, want_R=True, want_J=True):
        X = np.ascontiguousarray(X, dtype=np.float64)
        R = np.zeros(self.n_dofs) if want_R else None
        check(lib().mg_residual_and_jacobian(self.h, _p(X), _p(R), int(want_J)),
              "mg_residual_and_jacobian")
        return R

    def get_csr(self):
        rowptr = np.zeros(self.n_dofs + 1, dtype=np.int32)
        cols = np.zeros(self.nnz, dtype=np.int32)
        vals = np.zeros(self.nnz)
        check(lib().mg_get_csr(self.h, _p(rowptr), _p(cols), _p(vals)), "mg_get_csr")
        return rowptr, cols, vals

    def element_matrices(self, first, count, X=None):
        nd = {PHYS_HEX8: 24, PHYS_HEX8_NONLINEAR: 24, PHYS_MEMBRANE: 8, PHYS_HEAT: 4}[self.physics]
        Ke = np.zeros((count, nd, nd))
        fe = np.zeros((count, nd))
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        check(lib().mg_element_matrices(self.h, _p(Xa), first, count, _p(Ke), _p(fe)),
              "mg_element_matrices")
        return Ke, fe

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n_dofs)
        check(lib().mg_spmv(self.h, _p(x), _p(y)), "mg_spmv")
        return y

    def solve(self, opts=None, X=None, raise_on_error=True):
        o = opts if opts is not None else default_opts()
        Xa = np.zeros(self.n_dofs) if X is None else np.ascontiguousarray(X, dtype=np.float64).copy()
        rep = SolveReport()
        rc = lib().mg_solve(self.h, ctypes.byref(o), _p(Xa), ctypes.byref(rep))
        if raise_on_error:
            check(rc, "mg_solve")
        return Xa, rep

    def solve_resident(self, opts):
        """Solve with all inputs already on the device; the solution stays there."""
        rep = SolveReport()
        rc = lib().mg_solve(self.h, ctypes.byref(opts), None, ctypes.byref(rep))
        return rc, rep

    def matfree_apply(self, x, precision=MIXED_TF32):
        """One application of the mixed-precision operator (x zero on Dirichlet dofs)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n_dofs)
        check(lib().mg_debug_matfree_apply(self.h, precision, _p(x), _p(y)),
              "mg_debug_matfree_apply")
        return y

    def solution(self):
        X = np.zeros(self.n_dofs)
        check(lib().mg_get_solution(self.h, _p(X)), "mg_get_solution")
        return X

    def compliance(self, X=None, want_sens=True):
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        c = ctypes.c_double()
        dc = np.zeros(self.n_nodes if getattr(self, "nodal", False) else self.n_elems) if want_sens else None
        check(lib().mg_compliance(self.h, _p(Xa), ctypes.byref(c), _p(dc)), "mg_compliance")
        return c.value, dc

    def set_side_loads(self, elems, sides, values):
        """pressure on HEX8 faces / heat flux on QUAD4 edges (mg_set_side_loads)"""
        e = np.ascontiguousarray(elems, dtype=np.int32)
        s = np.ascontiguousarray(sides, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        if not (e.shape == s.shape == v.shape):
            raise ValueError("elems, sides and values must have one entry per side load")
        check(lib().mg_set_side_loads(self.h, e.shape[0], _p(e), _p(s), _p(v)), "mg_set_side_loads")

    def ks_stress(self, p_ks, sigma0, stress_penalty=0.0, X=None, want_sens=True):
        """KS-aggregated von Mises stress, the largest von Mises stress and (want_sens) the
        total density derivative of the KS value (mg_ks_stress)"""
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        q, vmax = ctypes.c_double(), ctypes.c_double()
        d = np.zeros(self.n_elems) if want_sens else None
        check(lib().mg_ks_stress(self.h, _p(Xa), p_ks, sigma0, stress_penalty, ctypes.byref(q),
                                 ctypes.byref(vmax), _p(d)), "mg_ks_stress")
        return q.value, vmax.value, d

    def adjoint_solve(self, X, rhs, opts=None):
        """lambda with J(X)^T lambda = rhs (mg_adjoint_solve)"""
        Xa = np.ascontiguousarray(X, dtype=np.float64)
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        lam = np.zeros(self.n_dofs)
        o = opts if opts is not None else default_opts()
        check(lib().mg_adjoint_solve(self.h, _p(Xa), _p(b), ctypes.byref(o), _p(lam)),
              "mg_adjoint_solve")
        return lam

    def mean_temperature(self, T=None, opts=None, want_sens=True):
        Ta = None if T is None else np.ascontiguousarray(T, dtype=np.float64)
        q, dk0 = ctypes.c_double(), ctypes.c_double()
        ds = np.zeros(self.n_elems) if want_sens else None
        o = opts if opts is not None else default_opts(krylov=KRYLOV_BICGSTAB)
        check(lib().mg_mean_temperature(self.h, _p(Ta), ctypes.byref(o), ctypes.byref(q),
                                        ctypes.byref(dk0) if want_sens else None, _p(ds)),
              "mg_mean_temperature")
        return q.value, (dk0.value if want_sens else None), ds

    def sensitivity_solve(self, X, kind, index=0, opts=None):
        """dX/dp with J(X) dX/dp = -dR/dp (mg_sensitivity_solve)"""
        Xa = np.ascontiguousarray(X, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        o = opts if opts is not None else default_opts()
        check(lib().mg_sensitivity_solve(self.h, _p(Xa), kind, index, ctypes.byref(o), _p(out)),
              "mg_sensitivity_solve")
        return out

    def output_derivative(self, output, X=None):
        """dq/dX of OUTPUT_COMPLIANCE / OUTPUT_MEAN_TEMPERATURE (mg_output_derivative)"""
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        check(lib().mg_output_derivative(self.h, output, _p(Xa), _p(out)), "mg_output_derivative")
        return out

    def element_calculations(self, elem, sol_elem, want_K=True):
        """element residual and Jacobian at a var-blocked element-local solution
        (mg_element_calculations)"""
        sol = np.ascontiguousarray(sol_elem, dtype=np.float64)
        nd = sol.shape[0]
        K = np.zeros((nd, nd)) if want_K else None
        f = np.zeros(nd)
        check(lib().mg_element_calculations(self.h, elem, _p(sol), _p(K), _p(f)),
              "mg_element_calculations")
        return f, K

    def element_sensitivity(self, elem, sol_elem, kind, index=0):
        sol = np.ascontiguousarray(sol_elem, dtype=np.float64)
        out = np.zeros(sol.shape[0])
        check(lib().mg_element_sensitivity(self.h, elem, _p(sol), kind, index, _p(out)),
              "mg_element_sensitivity")
        return out

    def sensitivity_assemble(self, kind, index=0, X=None):
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        check(lib().mg_sensitivity_assemble(self.h, _p(Xa), kind, index, _p(out)),
              "mg_sensitivity_assemble")
        return out


class Batch:
    """Batched SIMP design evaluations (mg_batch_*).  designs: list of dicts with
    keys nx, ny, nz, rho (nx*ny*nz densities) and either spans (list of (j0, j1)
    node ranges of the unit -z line load on the x = nx, z = 0 edge, one per load
    case) or F (n_cases x n_dofs nodal loads); optional node_fix."""

    def __init__(self, designs, material=None):
        L = lib()
        m = dict(SIMP_MATERIAL)
        m.update(material or {})
        self._mat = MaterialDesc(**m)
        self._keep = []
        arr = (BatchProblem * len(designs))()
        self.shapes = []
        for i, d in enumerate(designs):
            nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
            rho = np.ascontiguousarray(d["rho"], dtype=np.float64)
            bp = arr[i]
            bp.nx, bp.ny, bp.nz = nx, ny, nz
            bp.rho = rho.ctypes.data
            self._keep.append(rho)
            if d.get("F") is not None:
                F = np.ascontiguousarray(d["F"], dtype=np.float64).reshape(-1)
                nc = F.size // (3 * (nx + 1) * (ny + 1) * (nz + 1))
                bp.F = F.ctypes.data
                self._keep.append(F)
            else:
                sp = np.ascontiguousarray(np.asarray(d["spans"], dtype=np.int32).reshape(-1))
                nc = sp.size // 2
                bp.span = sp.ctypes.data
                self._keep.append(sp)
            bp.n_cases = nc
            if d.get("node_fix") is not None:
                nf = np.ascontiguousarray(d["node_fix"], dtype=np.uint8)
                bp.node_fix = nf.ctypes.data
                self._keep.append(nf)
            self.shapes.append((nx, ny, nz, nc))
        h = _vp()
        check(L.mg_batch_create(arr, len(designs), ctypes.byref(self._mat), ctypes.byref(h)),
              "mg_batch_create")
        self._keep = []
        self.h = h
        nd, npb, nl = _i32(), _i32(), _i32()
        ndof, nbytes = _i64(), _i64()
        check(L.mg_batch_info(self.h, ctypes.byref(nd), ctypes.byref(npb), ctypes.byref(ndof),
                              ctypes.byref(nl), ctypes.byref(nbytes)), "mg_batch_info")
        self.n_designs, self.n_problems, self.n_dofs = nd.value, npb.value, ndof.value
        self.n_levels, self.device_bytes = nl.value, nbytes.value

    def close(self):
        if getattr(self, "h", None):
            lib().mg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return lib().mg_batch_stream(self.h)

    def set_design(self, d, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        check(lib().mg_batch_set_design(self.h, d, _p(rho)), "mg_batch_set_design")

    def set_design_device(self, d, ptr):
        check(lib().mg_batch_set_design_device(self.h, d, ctypes.c_void_p(ptr)),
              "mg_batch_set_design_device")

    def solve(self, opts, active=None, raise_on_error=True):
        reps = (SolveReport * self.n_problems)()
        if active is None:
            rc = lib().mg_batch_solve(self.h, ctypes.byref(opts), reps)
        else:
            act = np.ascontiguousarray(active, dtype=np.uint8)
            rc = lib().mg_batch_solve_subset(self.h, ctypes.byref(opts), _p(act), reps)
        if raise_on_error:
            check(rc, "mg_batch_solve")
        return rc, list(reps)

    def results(self, d, want_u=False):
        nx, ny, nz, nc = self.shapes[d]
        ne = nx * ny * nz
        nd = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        comp = np.zeros(nc)
        dc = np.zeros((nc, ne))
        u = np.zeros((nc, nd)) if want_u else None
        check(lib().mg_batch_results(self.h, d, _p(comp), _p(dc), _p(u)), "mg_batch_results")
        return comp, dc, u

    def autotune(self, opts, max_trials=16):
        secs = ctypes.c_double()
        check(lib().mg_batch_autotune(self.h, ctypes.byref(opts), max_trials, ctypes.byref(secs)),
              "mg_batch_autotune")
        return opts, secs.value


class Filter:
    """Density filter (mg_filter_*): Filter.grid(nx, ny, nz, radius) over element
    centroids, or Filter(points, radius) over arbitrary points."""

    def __init__(self, points=None, radius=1.5, dv=None, _grid=None):
        h = _vp()
        self._dv = None if dv is None else np.ascontiguousarray(dv, dtype=np.uint8)
        if _grid is not None:
            nx, ny, nz, hx, hy, hz = _grid
            check(lib().mg_filter_create_grid(nx, ny, nz, hx, hy, hz, radius, _p(self._dv), ctypes.byref(h)),
                  "mg_filter_create_grid")
        else:
            pts = np.ascontiguousarray(points, dtype=np.float64)
            check(lib().mg_filter_create_points(pts.shape[0], pts.shape[1], _p(pts), radius, _p(self._dv),
                                                ctypes.byref(h)), "mg_filter_create_points")
        self.h = h
        n, nnz = _i64(), _i64()
        check(lib().mg_filter_info(self.h, ctypes.byref(n), ctypes.byref(nnz)), "mg_filter_info")
        self.n, self.nnz = n.value, nnz.value

    @classmethod
    def grid(cls, nx, ny, nz, radius, dv=None, h=(1.0, 1.0, 1.0)):
        return cls(radius=radius, dv=dv, _grid=(nx, ny, nz, h[0], h[1], h[2]))

    def apply(self, x, transpose=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        check(lib().mg_filter_apply(self.h, _p(x), _p(y), int(transpose)), "mg_filter_apply")
        return y

    def close(self):
        if getattr(self, "h", None):
            lib().mg_filter_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Request loop (mg_server_*): continuous batching of design evaluations."""

    def __init__(self, opts=None, hbm_cap_bytes=0, max_inflight=0, material=None):
        m = dict(SIMP_MATERIAL)
        m.update(material or {})
        self._mat = MaterialDesc(**m)
        so = ServerOpts()
        so.hbm_cap_bytes = hbm_cap_bytes
        so.solve = opts if opts is not None else default_opts(precision=MIXED_TF32X3, rtol=1e-8,
                                                                inner_rtol=1e-3)
        so.max_inflight = max_inflight
        self._opts = so
        h = _vp()
        check(lib().mg_server_create(ctypes.byref(self._mat), ctypes.byref(so), ctypes.byref(h)),
              "mg_server_create")
        self.h = h
        self._out = {}

    def close(self):
        if getattr(self, "h", None):
            lib().mg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, tag, chain, nx, ny, nz, rho, spans, want_dc=True, arrival_s=0.0):
        """Returns (compliance, dc) output arrays, filled when the completion posts."""
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        sp = np.ascontiguousarray(np.asarray(spans, dtype=np.int32).reshape(-1))
        nc = sp.size // 2
        comp = np.zeros(nc)
        dc = np.zeros((nc, nx * ny * nz)) if want_dc else None
        q = Request(chain=chain, nx=nx, ny=ny, nz=nz, n_cases=nc, rho=rho.ctypes.data,
                    span=sp.ctypes.data, compliance_out=comp.ctypes.data,
                    dc_out=None if dc is None else dc.ctypes.data, arrival_s=arrival_s, tag=tag)
        self._out[tag] = (comp, dc)  # keep the output buffers alive until posted
        check(lib().mg_server_submit(self.h, ctypes.byref(q)), "mg_server_submit")
        return comp, dc

    def poll(self, max_n=1024, timeout_s=0.0):
        buf = (Completion * max_n)()
        n = _i32()
        check(lib().mg_server_poll(self.h, buf, max_n, ctypes.byref(n), timeout_s), "mg_server_poll")
        return [buf[i] for i in range(n.value)]

    def drain(self, timeout_s=0.0):
        check(lib().mg_server_drain(self.h, timeout_s), "mg_server_drain")

    def stats(self):
        st = ServerStats()
        check(lib().mg_server_get_stats(self.h, ctypes.byref(st)), "mg_server_get_stats")
        return st.as_dict()

    def run_synthetic(self, n_requests, rate, n_chains=64, sizes=None, big=(192, 96, 96),
                      big_fraction=0.02, max_cases=4, noise=0.02, seed=0):
        d = synthetic_desc(n_requests, rate, n_chains, sizes, big, big_fraction, max_cases, noise, seed)
        comp = np.zeros((n_requests, max_cases))
        st = ServerStats()
        check(lib().mg_server_run_synthetic(self.h, ctypes.byref(d), _p(comp), ctypes.byref(st)),
              "mg_server_run_synthetic")
        return st.as_dict(), comp


def synthetic_desc(n_requests, rate, n_chains=64, sizes=None, big=(192, 96, 96), big_fraction=0.02,
                   max_cases=4, noise=0.02, seed=0):
    """The mg_synthetic_desc of Server.run_synthetic with the same arguments (the sizes
    array is kept alive on the returned object)."""
    sizes = BATCH_SIZES if sizes is None else sizes
    sz = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32).reshape(-1))
    d = SyntheticDesc(n_requests=n_requests, rate=rate, n_chains=n_chains, n_sizes=sz.size // 3,
                      sizes=sz.ctypes.data, big_fraction=big_fraction, big_nx=big[0], big_ny=big[1],
                      big_nz=big[2], max_cases=max_cases, noise=noise, seed=seed)
    d._sizes = sz
    return d


def synthetic_request(desc, index, want_rho=True):
    """Request `index` of a synthetic stream (mg_server_synthetic_request): dict with
    chain, grid, spans and (want_rho) the densities that run_synthetic submitted."""
    info = np.zeros(5, dtype=np.int32)
    check(lib().mg_server_synthetic_request(ctypes.byref(desc), index, _p(info), None, None),
          "mg_server_synthetic_request")
    span = np.zeros(2 * int(info[4]), dtype=np.int32)
    rho = np.zeros(int(info[1]) * int(info[2]) * int(info[3])) if want_rho else None
    check(lib().mg_server_synthetic_request(ctypes.byref(desc), index, _p(info), _p(span), _p(rho)),
          "mg_server_synthetic_request")
    return {"chain": int(info[0]), "grid": (int(info[1]), int(info[2]), int(info[3])),
            "spans": [(int(span[2 * k]), int(span[2 * k + 1])) for k in range(int(info[4]))],
            "rho": rho}


# ------------------------------------------------------------------ benchmark problems
SIMP_MATERIAL = dict(E0=1.0, Emin=1e-9, nu=0.3, penal=3.0, thickness=1.0, k0=0.0, k_beta=0.0)


def simp_cantilever(nx, ny, nz, load_y0=0, load_y1=None, material=None, physics=PHYS_HEX8,
                    load=1.0):
    """HEX8 SIMP cantilever: x=0 face clamped, total -z load (magnitude `load`) spread
    over the nodes of the z=0 edge at x=max between node rows load_y0..load_y1.
    physics PHYS_HEX8_NONLINEAR gives the Green-Lagrange (large-deflection) form."""
    coords, conn = grid_hex8(nx, ny, nz)
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    k, j = np.meshgrid(np.arange(NZ), np.arange(NY), indexing="ij")
    clamp = (NX * (j + NY * k)).reshape(-1)
    fixed = (clamp[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    y1 = ny if load_y1 is None else load_y1
    ys = np.arange(load_y0, y1 + 1)
    load_nodes = nx + NX * ys
    load_dofs = load_nodes * 3 + 2
    load_vals = np.full(ys.shape[0], -float(load) / ys.shape[0])
    return Problem(physics, coords, conn, material or SIMP_MATERIAL, fixed_dofs=fixed,
                   load_dofs=load_dofs, load_values=load_vals, grid=(nx, ny, nz))


def read_bdf(path=None, text=None, dpn=3):
    """Nastran bulk data mesh (mg_bdf_read / mg_bdf_parse): dict with coords
    (n x 3), conn (n_elems x npe, node indices), grid_ids, elem_ids, pids,
    fixed_dofs and (load_dofs, load_values) for dpn dofs per node."""
    L = lib()
    h = _vp()
    if text is not None:
        b = text.encode() if isinstance(text, str) else bytes(text)
        check(L.mg_bdf_parse(b, len(b), ctypes.byref(h)), "mg_bdf_parse")
    else:
        check(L.mg_bdf_read(os.fsencode(path), ctypes.byref(h)), "mg_bdf_read")
    try:
        nn, ne, npe = _i64(), _i64(), _i32()
        check(L.mg_bdf_sizes(h, ctypes.byref(nn), ctypes.byref(ne), ctypes.byref(npe)), "mg_bdf_sizes")
        coords = np.zeros((nn.value, 3))
        gids = np.zeros(nn.value, dtype=np.int64)
        check(L.mg_bdf_nodes(h, _p(coords), _p(gids)), "mg_bdf_nodes")
        conn = np.zeros((ne.value, npe.value), dtype=np.int32)
        eids = np.zeros(ne.value, dtype=np.int64)
        pids = np.zeros(ne.value, dtype=np.int32)
        check(L.mg_bdf_elements(h, _p(conn), _p(eids), _p(pids)), "mg_bdf_elements")
        n = _i64()
        check(L.mg_bdf_constraints(h, dpn, None, ctypes.byref(n)), "mg_bdf_constraints")
        fixed = np.zeros(n.value, dtype=np.int64)
        check(L.mg_bdf_constraints(h, dpn, _p(fixed), ctypes.byref(n)), "mg_bdf_constraints")
        check(L.mg_bdf_loads(h, dpn, None, None, ctypes.byref(n)), "mg_bdf_loads")
        ld = np.zeros(n.value, dtype=np.int64)
        lv = np.zeros(n.value)
        check(L.mg_bdf_loads(h, dpn, _p(ld), _p(lv), ctypes.byref(n)), "mg_bdf_loads")
    finally:
        L.mg_bdf_destroy(h)
    return dict(coords=coords, conn=conn, grid_ids=gids, elem_ids=eids, pids=pids, fixed_dofs=fixed,
                load_dofs=ld, load_values=lv)


def write_exodus(path, coords, conn, nodal=None, elem=None, title=None, time=0.0):
    """One time step of a HEX8 / QUAD4 mesh with nodal and element fields
    (dicts name -> array) as an ExodusII file (mg_exodus_write)."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nodal = nodal or {}
    elem = elem or {}
    nn, dim = coords.shape
    ne, npe = conn.shape
    nn_names = (ctypes.c_char_p * max(1, len(nodal)))(*[k.encode() for k in nodal])
    ne_names = (ctypes.c_char_p * max(1, len(elem)))(*[k.encode() for k in elem])
    nv = np.ascontiguousarray(np.array([np.asarray(v, np.float64).reshape(nn) for v in nodal.values()]).reshape(-1))
    ev = np.ascontiguousarray(np.array([np.asarray(v, np.float64).reshape(ne) for v in elem.values()]).reshape(-1))
    check(lib().mg_exodus_write(os.fsencode(path), (title or "").encode(), dim, npe, nn, _p(coords), ne, _p(conn),
                                len(nodal), nn_names, _p(nv) if nodal else None, len(elem), ne_names,
                                _p(ev) if elem else None, float(time)), "mg_exodus_write")


def read_exodus(path):
    """Mesh of an ExodusII file (mg_exodus_read_mesh): coords (n x dim) and conn
    (n_elems x nodes per element, 0-based) of every element block."""
    L = lib()
    dim, npe, nn, ne = _i32(), _i32(), _i64(), _i64()
    check(L.mg_exodus_read_sizes(os.fsencode(path), ctypes.byref(dim), ctypes.byref(npe), ctypes.byref(nn),
                                 ctypes.byref(ne)), "mg_exodus_read_sizes")
    coords = np.zeros((nn.value, dim.value))
    conn = np.zeros((ne.value, npe.value), dtype=np.int32)
    check(L.mg_exodus_read_mesh(os.fsencode(path), _p(coords), _p(conn)), "mg_exodus_read_mesh")
    return coords, conn


BATCH_SIZES = ((16, 8, 8), (32, 16, 16), (48, 24, 24), (64, 32, 32), (96, 48, 48))


def batch_designs(n, seed=0, sizes=BATCH_SIZES, max_cases=4):
    """Seeded batch of SIMP cantilever designs: grid drawn uniformly from `sizes`,
    densities iid U[0.01, 1], 1..max_cases load cases, each a unit -z line load on
    the x = max, z = 0 edge over a random contiguous node span along y."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, ny, nz = sizes[int(rng.integers(len(sizes)))]
        rho = rng.uniform(0.01, 1.0, nx * ny * nz)
        nc = int(rng.integers(1, max_cases + 1))
        spans = []
        for _ in range(nc):
            j0 = int(rng.integers(0, ny + 1))
            j1 = int(rng.integers(j0, ny + 1))
            spans.append((j0, j1))
        out.append(dict(nx=nx, ny=ny, nz=nz, rho=rho, spans=spans))
    return out


def heat_square(nx=200, ny=200, k0=1.0, beta=0.01, h=1.0, hc=10.0, Tinf=0.0, q=1.0,
                lo=0.25, hi=0.75):
    """QUAD4 conduction on [0,1]^2: T=0 at x=0, convection on x=1, source q on
    the element-aligned box [lo,hi]^2."""
    coords, conn = grid_quad4(nx, ny)
    NX = nx + 1
    fixed = (NX * np.arange(ny + 1)).astype(np.int64)
    conv_elems = (nx - 1) + nx * np.arange(ny)
    conv_sides = np.ones(ny, dtype=np.int32)
    ic = (np.arange(nx) + 0.5) / nx
    jc = (np.arange(ny) + 0.5) / ny
    inside = ((jc[:, None] > lo) & (jc[:, None] < hi)) & ((ic[None, :] > lo) & (ic[None, :] < hi))
    src = np.where(inside, q, 0.0).reshape(-1)
    mat = dict(E0=0.0, Emin=0.0, nu=0.0, penal=1.0, thickness=h, k0=k0, k_beta=beta)
    return Problem(PHYS_HEAT, coords, conn, mat, fixed_dofs=fixed, conv_elems=conv_elems,
                   conv_sides=conv_sides, conv_h=hc, conv_Tinf=Tinf, source_elem=src,
                   grid=(nx, ny, 0))


def device_info():
    name = ctypes.create_string_buffer(256)
    sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().mg_device_info(name, 256, ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi)),
          "mg_device_info")
    return dict(name=name.value.decode(), sm_count=sm.value, cc=(ma.value, mi.value))
