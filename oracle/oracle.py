"""ctypes binding of the FP64 CPU oracle (oracle/mast_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the reference its results are compared with, and by bench.py's CPU-baseline
arm.  The product library never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmastoracle.so")

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


class SimpDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("E0", ctypes.c_double), ("Emin", ctypes.c_double), ("nu", ctypes.c_double),
                ("penal", ctypes.c_double), ("load_y0", ctypes.c_int), ("load_y1", ctypes.c_int),
                ("load_total", ctypes.c_double), ("rtol", ctypes.c_double), ("maxit", ctypes.c_int)]


class SimpReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("relres", ctypes.c_double),
                ("compliance", ctypes.c_double), ("t_assemble", ctypes.c_double),
                ("t_solve", ctypes.c_double), ("t_sens", ctypes.c_double)]


class HeatDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("lx", ctypes.c_double),
                ("ly", ctypes.c_double), ("k0", ctypes.c_double), ("beta", ctypes.c_double),
                ("h", ctypes.c_double), ("hc", ctypes.c_double), ("Tinf", ctypes.c_double),
                ("rtol", ctypes.c_double), ("newton_rtol", ctypes.c_double),
                ("maxit", ctypes.c_int), ("max_newton", ctypes.c_int),
                ("consistent", ctypes.c_int), ("krylov", ctypes.c_int)]


class HeatReport(ctypes.Structure):
    _fields_ = [("newton_iterations", ctypes.c_int), ("krylov_iterations", ctypes.c_int),
                ("residual_norm", ctypes.c_double), ("mean_temperature", ctypes.c_double),
                ("dq_dk0", ctypes.c_double), ("t_total", ctypes.c_double)]


def build(force=False):
    """Compile the oracle with its Makefile (gcc -O3 -fopenmp)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "mast_oracle.c")):
        subprocess.run(["make", "-B" if force else "all"], cwd=HERE, check=True,
                       stdout=subprocess.DEVNULL)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i64, i32, d, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        L.or_iso_stiffness_3d.argtypes = [d, d, _f64p]
        L.or_iso_stiffness_2d.argtypes = [d, d, i32, _f64p]
        L.or_hex8_shape.argtypes = [_f64p, _f64p, _f64p]
        L.or_quad4_shape.argtypes = [_f64p, _f64p, _f64p]
        L.or_hex8_internal.argtypes = [_f64p, d, d, _f64p, _f64p, vp]
        L.or_hex8_internal_sens.argtypes = [_f64p, d, d, _f64p, _f64p]
        L.or_hex8_internal_gl.argtypes = [_f64p, d, d, _f64p, _f64p, ctypes.c_void_p]
        L.or_hex8_stress.argtypes = [_f64p, d, d, _f64p, i32, _f64p, _f64p, _f64p, vp]
        L.or_hex8_pressure.argtypes = [_f64p, i32, d, _f64p]
        L.or_hex8_pressure.restype = None
        L.or_quad4_heat_flux.argtypes = [_f64p, i32, d, d, _f64p]
        L.or_quad4_heat_flux.restype = None
        L.or_quad4_membrane_internal.argtypes = [_f64p, d, d, d, _f64p, _f64p, vp]
        L.or_quad4_heat_internal.argtypes = [_f64p, d, d, d, d, _f64p, i32, _f64p, vp]
        L.or_quad4_heat_internal_sens.argtypes = [_f64p, d, d, d, _f64p, _f64p]
        L.or_quad4_heat_convection.argtypes = [_f64p, i32, d, d, d, _f64p, _f64p, vp]
        L.or_quad4_heat_source.argtypes = [_f64p, d, d, _f64p]
        L.or_grid_hex8.argtypes = [i32, i32, i32, d, d, d, _f64p, _i32p]
        L.or_grid_quad4.argtypes = [i32, i32, d, d, _f64p, _i32p]
        L.or_csr_pattern.argtypes = [i32, i32, i64, i64, _i32p, _i32p, vp]
        L.or_csr_pattern.restype = i64
        L.or_color_elements.argtypes = [i32, i64, i64, _i32p, _i32p]
        L.or_csr_spmv.argtypes = [i64, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.or_assemble_hex8.argtypes = [i64, i64, _f64p, _i32p, _f64p, d, _i32p, _i32p, _f64p,
                                       vp, i32, vp]
        L.or_assemble_quad4_membrane.argtypes = [i64, i64, _f64p, _i32p, _f64p, d, d, _i32p,
                                                 _i32p, _f64p, vp]
        L.or_assemble_quad4_heat.argtypes = [i64, i64, _f64p, _i32p, d, d, vp, d, vp, i64, vp,
                                             vp, d, d, _f64p, i32, _i32p, _i32p, vp, vp, vp]
        L.or_assemble_hex8_gl.argtypes = [i64, i64, _f64p, _i32p, _f64p, d, _f64p, vp, _i32p,
                                          _i32p, vp, vp, vp]
        L.or_pcg.argtypes = [i64, _i32p, _i32p, _f64p, _f64p, _f64p, d, i32,
                             ctypes.POINTER(d)]
        L.or_bicgstab.argtypes = L.or_pcg.argtypes
        L.or_simp_solve.argtypes = [ctypes.POINTER(SimpDesc), _f64p, _f64p, vp,
                                    ctypes.POINTER(SimpReport)]
        L.or_simp_solve_nodal.argtypes = [ctypes.POINTER(SimpDesc), _f64p, _f64p, vp,
                                          ctypes.POINTER(SimpReport)]
        L.or_simp_nodal_modulus.argtypes = [ctypes.POINTER(SimpDesc), i64, _i32p, _f64p, vp, vp]
        L.or_hex8_internal_qp.argtypes = [_f64p, _f64p, d, _f64p, _f64p, vp]
        L.or_simp_load_vector.argtypes = [ctypes.POINTER(SimpDesc), _f64p]
        L.or_simp_fixed_mask.argtypes = [ctypes.POINTER(SimpDesc), _u8p]
        L.or_simp_modulus.argtypes = [ctypes.POINTER(SimpDesc), i64, _f64p, vp, vp]
        L.or_heat_solve.argtypes = [ctypes.POINTER(HeatDesc), vp, vp, _f64p, vp,
                                    ctypes.POINTER(HeatReport)]
        L.or_filter_points.argtypes = [i64, i32, _f64p, d, vp, _f64p, _f64p, i32]
        L.or_grid_centroids.argtypes = [i32, i32, i32, d, d, d, _f64p]
        L.or_wtime.restype = d
        L.or_max_threads.restype = i32
        L.or_set_threads.argtypes = [i32]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------- element level
def iso_stiffness_3d(E, nu):
    C = np.zeros(36)
    lib().or_iso_stiffness_3d(E, nu, C)
    return C.reshape(6, 6)


def iso_stiffness_2d(E, nu, plane_stress=True):
    C = np.zeros(9)
    lib().or_iso_stiffness_2d(E, nu, int(plane_stress), C)
    return C.reshape(3, 3)


def hex8_internal(X, E, nu, u=None, want_K=True):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(24)
    u = np.zeros(24) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    f = np.zeros(24)
    K = np.zeros(576) if want_K else None
    rc = lib().or_hex8_internal(X, E, nu, u, f, _ptr(K))
    if rc:
        raise ValueError("degenerate HEX8 element")
    return f, (K.reshape(24, 24) if want_K else None)


def hex8_internal_gl(X, E, nu, u, want_K=True):
    """Green-Lagrange (total Lagrangian) HEX8 residual and tangent, var-blocked dofs."""
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(24)
    u = np.ascontiguousarray(u, dtype=np.float64)
    f = np.zeros(24)
    K = np.zeros(576) if want_K else None
    if lib().or_hex8_internal_gl(X, E, nu, u, f, _ptr(K)):
        raise ValueError("degenerate HEX8 element")
    return f, (K.reshape(24, 24) if want_K else None)


def hex8_internal_sens(X, dE, nu, u):
    df = np.zeros(24)
    lib().or_hex8_internal_sens(np.ascontiguousarray(X, dtype=np.float64).reshape(24), dE, nu,
                                np.ascontiguousarray(u, dtype=np.float64), df)
    return df


def quad4_membrane_internal(X, E, nu, h, u=None, want_K=True):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(8)
    u = np.zeros(8) if u is None else np.ascontiguousarray(u, dtype=np.float64)
    f = np.zeros(8)
    K = np.zeros(64) if want_K else None
    if lib().or_quad4_membrane_internal(X, E, nu, h, u, f, _ptr(K)):
        raise ValueError("degenerate QUAD4 element")
    return f, (K.reshape(8, 8) if want_K else None)


def quad4_heat_internal(X, k0, beta, s, h, T, consistent=True, want_K=True):
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(8)
    T = np.ascontiguousarray(T, dtype=np.float64)
    f = np.zeros(4)
    K = np.zeros(16) if want_K else None
    lib().or_quad4_heat_internal(X, k0, beta, s, h, T, int(consistent), f, _ptr(K))
    return f, (K.reshape(4, 4) if want_K else None)


def quad4_heat_convection(X, side, hc, Tinf, th, T):
    f = np.zeros(4)
    K = np.zeros(16)
    lib().or_quad4_heat_convection(np.ascontiguousarray(X, dtype=np.float64).reshape(8), side,
                                   hc, Tinf, th, np.ascontiguousarray(T, dtype=np.float64), f,
                                   _ptr(K))
    return f, K.reshape(4, 4)


def quad4_heat_source(X, q, th):
    f = np.zeros(4)
    lib().or_quad4_heat_source(np.ascontiguousarray(X, dtype=np.float64).reshape(8), q, th, f)
    return f


# ---------------------------------------------------------------- meshes / sparse
def grid_hex8(nx, ny, nz, lx=None, ly=None, lz=None):
    lx = float(nx if lx is None else lx)
    ly = float(ny if ly is None else ly)
    lz = float(nz if lz is None else lz)
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    coords = np.zeros(nn * 3)
    conn = np.zeros(nx * ny * nz * 8, dtype=np.int32)
    lib().or_grid_hex8(nx, ny, nz, lx, ly, lz, coords, conn)
    return coords.reshape(nn, 3), conn.reshape(-1, 8)


def grid_quad4(nx, ny, lx=1.0, ly=1.0):
    nn = (nx + 1) * (ny + 1)
    coords = np.zeros(nn * 2)
    conn = np.zeros(nx * ny * 4, dtype=np.int32)
    lib().or_grid_quad4(nx, ny, lx, ly, coords, conn)
    return coords.reshape(nn, 2), conn.reshape(-1, 4)


def csr_pattern(conn, n_nodes, dpn):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    npe = conn.shape[1]
    rowptr = np.zeros(n_nodes * dpn + 1, dtype=np.int32)
    nnz = lib().or_csr_pattern(npe, dpn, n_nodes, conn.shape[0], conn.reshape(-1), rowptr, None)
    cols = np.zeros(nnz, dtype=np.int32)
    lib().or_csr_pattern(npe, dpn, n_nodes, conn.shape[0], conn.reshape(-1), rowptr,
                         _ptr(cols))
    return rowptr, cols


def color_elements(conn, n_nodes):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    color = np.zeros(conn.shape[0], dtype=np.int32)
    nc = lib().or_color_elements(conn.shape[1], n_nodes, conn.shape[0], conn.reshape(-1), color)
    return nc, color


def assemble_hex8(coords, conn, E_elem, nu, rowptr, cols, fixed=None):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nc, color = color_elements(conn, coords.shape[0])
    vals = np.zeros(cols.shape[0])
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
    rc = lib().or_assemble_hex8(coords.shape[0], conn.shape[0], coords.reshape(-1),
                                conn.reshape(-1), np.ascontiguousarray(E_elem, dtype=np.float64),
                                nu, rowptr, cols, vals, _ptr(fx), nc, _ptr(color))
    if rc:
        raise ValueError("degenerate element in assembly")
    return vals


def assemble_quad4_membrane(coords, conn, E_elem, nu, h, rowptr, cols, fixed=None):
    """Linear QUAD4 membrane stiffness (2 dofs per node, node-interleaved) into the CSR
    pattern of csr_pattern(conn, n_nodes, 2); Dirichlet rows and columns eliminated."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    vals = np.zeros(cols.shape[0])
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
    rc = lib().or_assemble_quad4_membrane(coords.shape[0], conn.shape[0], coords.reshape(-1),
                                          conn.reshape(-1),
                                          np.ascontiguousarray(E_elem, dtype=np.float64), nu, h,
                                          rowptr, cols, vals, _ptr(fx))
    if rc:
        raise ValueError("degenerate element in assembly")
    return vals


def assemble_quad4_heat(coords, conn, k0, beta, s_elem, h, q_elem, conv_elem, conv_side, hc,
                        Tinf, T, consistent, rowptr, cols, fixed):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    n = coords.shape[0]
    vals = np.zeros(cols.shape[0])
    R = np.zeros(n)
    ce = np.ascontiguousarray(conv_elem, dtype=np.int32)
    cs = np.ascontiguousarray(conv_side, dtype=np.int32)
    s = None if s_elem is None else np.ascontiguousarray(s_elem, dtype=np.float64)
    q = None if q_elem is None else np.ascontiguousarray(q_elem, dtype=np.float64)
    fx = np.ascontiguousarray(fixed, dtype=np.uint8)
    lib().or_assemble_quad4_heat(n, conn.shape[0], coords.reshape(-1), conn.reshape(-1), k0,
                                 beta, _ptr(s), h, _ptr(q), ce.shape[0], _ptr(ce), _ptr(cs), hc,
                                 Tinf, np.ascontiguousarray(T, dtype=np.float64),
                                 int(consistent), rowptr, cols, _ptr(vals), _ptr(R), _ptr(fx))
    return vals, R


def assemble_hex8_gl(coords, conn, E_elem, nu, u, F, rowptr, cols, fixed, want_K=True):
    """Green-Lagrange HEX8 system at u: (CSR values of the tangent or None, R = f_int - F)."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    n = coords.shape[0] * 3
    vals = np.zeros(cols.shape[0]) if want_K else None
    R = np.zeros(n)
    Fv = None if F is None else np.ascontiguousarray(F, dtype=np.float64)
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
    if lib().or_assemble_hex8_gl(coords.shape[0], conn.shape[0], coords.reshape(-1),
                                 conn.reshape(-1), np.ascontiguousarray(E_elem, dtype=np.float64),
                                 nu, np.ascontiguousarray(u, dtype=np.float64), _ptr(Fv), rowptr,
                                 cols, _ptr(vals), _ptr(R), _ptr(fx)):
        raise ValueError("degenerate element in assembly")
    return vals, R


def newton_hex8_gl(coords, conn, E_elem, nu, F, fixed, rtol=1e-10, max_newton=30,
                   krylov_rtol=1e-13):
    """NonlinearSystem::solve under Newton (src/base/nonlinear_system.cpp:209-235):
    J du = R, u -= du until ||R|| <= rtol ||R0||.  Returns u and the ||R|| history."""
    rowptr, cols = csr_pattern(conn, coords.shape[0], 3)
    u = np.zeros(coords.shape[0] * 3)
    hist = []
    for _ in range(max_newton + 1):
        vals, R = assemble_hex8_gl(coords, conn, E_elem, nu, u, F, rowptr, cols, fixed)
        hist.append(float(np.linalg.norm(R)))
        if hist[-1] <= rtol * hist[0] or hist[-1] == 0.0 or len(hist) > max_newton:
            break
        du, _, _ = pcg(rowptr, cols, vals, R, krylov_rtol, 100000)
        u -= du
    return u, hist


def hex8_gl_compliance_sens(coords, conn, dE_elem, nu, u, E_elem, F, fixed):
    """Adjoint density sensitivity of C = F.u at the equilibrium u of the Green-Lagrange
    system (AssemblyBase::calculate_output_adjoint_sensitivity, assembly_base.cpp:555-590):
    K_T(u) lambda = F, dC/drho_e = -dE_e lambda_e . f1_e(u), f1 the unit-modulus force."""
    rowptr, cols = csr_pattern(conn, coords.shape[0], 3)
    vals, _ = assemble_hex8_gl(coords, conn, E_elem, nu, u, F, rowptr, cols, fixed)
    lam, _, _ = pcg(rowptr, cols, vals, np.where(np.asarray(fixed) == 1, 0.0, F), 1e-14, 100000)
    dc = np.zeros(conn.shape[0])
    for e in range(conn.shape[0]):
        ue = u.reshape(-1, 3)[conn[e]].T.reshape(-1)
        le = lam.reshape(-1, 3)[conn[e]].T.reshape(-1)
        f1, _ = hex8_internal_gl(coords[conn[e]], 1.0, nu, ue, want_K=False)
        dc[e] = -dE_elem[e] * float(le @ f1)
    return dc


def hex8_pressure(X, side, p):
    """external load (var-blocked) of pressure p on HEX8 side `side`"""
    f = np.zeros(24)
    lib().or_hex8_pressure(np.ascontiguousarray(X, dtype=np.float64).reshape(24), side, p, f)
    return f


def quad4_heat_flux(X, side, flux, th):
    """residual contribution of an outward heat flux on QUAD4 side `side`"""
    f = np.zeros(4)
    lib().or_quad4_heat_flux(np.ascontiguousarray(X, dtype=np.float64).reshape(8), side, flux, th, f)
    return f


def hex8_stress(X, E, nu, u, nonlinear=False, want_dsig=False):
    """Gauss-point stress (8, 6), von Mises (8), JxW (8) and d sigma / d u (8, 6, 24)."""
    sig, vm, jxw = np.zeros(48), np.zeros(8), np.zeros(8)
    ds = np.zeros(8 * 6 * 24) if want_dsig else None
    if lib().or_hex8_stress(np.ascontiguousarray(X, dtype=np.float64).reshape(24), E, nu,
                            np.ascontiguousarray(u, dtype=np.float64), int(nonlinear), sig, vm,
                            jxw, _ptr(ds)):
        raise ValueError("degenerate HEX8 element")
    return sig.reshape(8, 6), vm, jxw, (ds.reshape(8, 6, 24) if want_dsig else None)


def _dvm_dsig(s):
    """d sigma_vm / d sigma (Voigt), zero where sigma_vm = 0
    (StressStrainOutputBase::Data::dvon_Mises_stress_dX, stress_output_base.cpp:199-233)."""
    P = 0.5 * ((s[0] - s[1]) ** 2 + (s[1] - s[2]) ** 2 + (s[2] - s[0]) ** 2) + \
        3.0 * (s[3] ** 2 + s[4] ** 2 + s[5] ** 2)
    if not P > 0.0:
        return np.zeros(6)
    return 0.5 / np.sqrt(P) * np.array([2 * s[0] - s[1] - s[2], 2 * s[1] - s[2] - s[0],
                                        2 * s[2] - s[0] - s[1], 6 * s[3], 6 * s[4], 6 * s[5]])


def ks_stress(coords, conn, Es_elem, dEs_elem, nu, u, p_ks, sigma0, nonlinear=False):
    """KSStressStrainOutput over every element (ks_stress_output.cpp:41-99, 117-151, 196-246):
    q = ln(sum_qp exp(p (vm - s0)/s0) JxW / sum_qp JxW) / p with the stress of the modulus
    Es (the stress penalty of example_6.cpp:579-592).  Returns q, max vm, dq/du (global,
    node-interleaved) and the direct partial dq/drho_e (through Es at fixed u)."""
    n_el = conn.shape[0]
    w_all, jxw_all, vm_all, sig_all, dsig_all = [], [], [], [], []
    for e in range(n_el):
        ue = u.reshape(-1, 3)[conn[e]].T.reshape(-1)
        sig, vm, jxw, ds = hex8_stress(coords[conn[e]], Es_elem[e], nu, ue, nonlinear, True)
        vm_all.append(vm)
        jxw_all.append(jxw)
        sig_all.append(sig)
        dsig_all.append(ds)
    vm_all, jxw_all = np.array(vm_all), np.array(jxw_all)
    w = np.exp(p_ks * (vm_all - sigma0) / sigma0) * jxw_all
    I, V = w.sum(), jxw_all.sum()
    q = np.log(I / V) / p_ks
    dq_du = np.zeros(u.shape[0])
    for e in range(n_el):
        ge = np.zeros(24)
        for qp in range(8):
            ge += (_dvm_dsig(sig_all[e][qp]) @ dsig_all[e][qp]) * w[e, qp]
        ge /= sigma0 * I
        for a in range(8):
            for i in range(3):
                dq_du[conn[e][a] * 3 + i] += ge[i * 8 + a]
    dq_drho = (dEs_elem / Es_elem) * (vm_all * w).sum(axis=1) / (sigma0 * I)
    return q, vm_all.max(), dq_du, dq_drho


def ks_stress_total_sensitivity(coords, conn, E_elem, dE_elem, Es_elem, dEs_elem, nu, u, fixed,
                                p_ks, sigma0, nonlinear=False):
    """dq/drho_e = partial + lambda . dR/drho_e with K(u)^T lambda = -dq/du
    (example_6.cpp:798-874: adjoint_solve, then the adjoint term g1 at the solve's penalty
    and the direct term g2 at the stress penalty)."""
    q, vmax, dq_du, dq_drho = ks_stress(coords, conn, Es_elem, dEs_elem, nu, u, p_ks, sigma0,
                                        nonlinear)
    rowptr, cols = csr_pattern(conn, coords.shape[0], 3)
    if nonlinear:
        vals, _ = assemble_hex8_gl(coords, conn, E_elem, nu, u, None, rowptr, cols, fixed)
    else:
        vals = assemble_hex8(coords, conn, E_elem, nu, rowptr, cols, fixed)
    rhs = np.where(np.asarray(fixed) == 1, 0.0, -dq_du)
    lam, _, _ = pcg(rowptr, cols, vals, rhs, 1e-14, 100000)
    total = dq_drho.copy()
    for e in range(conn.shape[0]):
        ue = u.reshape(-1, 3)[conn[e]].T.reshape(-1)
        le = lam.reshape(-1, 3)[conn[e]].T.reshape(-1)
        if nonlinear:
            f1, _ = hex8_internal_gl(coords[conn[e]], 1.0, nu, ue, want_K=False)
        else:
            _, K1 = hex8_internal(coords[conn[e]], 1.0, nu)
            f1 = K1 @ ue
        total[e] += dE_elem[e] * float(le @ f1)
    return q, vmax, total


def spmv(rowptr, cols, vals, x):
    y = np.zeros(rowptr.shape[0] - 1)
    lib().or_csr_spmv(y.shape[0], rowptr, cols, vals, np.ascontiguousarray(x, np.float64), y)
    return y


def pcg(rowptr, cols, vals, b, rtol, maxit, x0=None):
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    rr = ctypes.c_double(0)
    it = lib().or_pcg(n, rowptr, cols, vals, np.ascontiguousarray(b, np.float64), x, rtol,
                      maxit, ctypes.byref(rr))
    return x, it, rr.value


# ---------------------------------------------------------------- pipelines
def simp_desc(nx, ny, nz, E0=1.0, Emin=1e-9, nu=0.3, penal=3.0, load_y0=0, load_y1=None,
              rtol=1e-10, maxit=200000):
    return SimpDesc(nx, ny, nz, E0, Emin, nu, penal, load_y0, ny if load_y1 is None else load_y1,
                    1.0, rtol, maxit)


def simp_solve(desc, rho, want_sens=True):
    n_el = desc.nx * desc.ny * desc.nz
    n = (desc.nx + 1) * (desc.ny + 1) * (desc.nz + 1) * 3
    u = np.zeros(n)
    dc = np.zeros(n_el) if want_sens else None
    rep = SimpReport()
    rc = lib().or_simp_solve(ctypes.byref(desc), np.ascontiguousarray(rho, np.float64), u,
                             _ptr(dc), ctypes.byref(rep))
    if rc:
        raise RuntimeError("oracle SIMP solve failed (%d)" % rc)
    return u, dc, rep


def simp_solve_nodal(desc, rho_nodes, want_sens=True):
    """The ex-6 sequence with a nodal density field (MeshFieldFunction over a
    FIRST-order LAGRANGE "rho", example_6.cpp:104-137, 250-252): the modulus at
    each Gauss point from the trilinear density there; dc per node."""
    n_nodes = (desc.nx + 1) * (desc.ny + 1) * (desc.nz + 1)
    u = np.zeros(3 * n_nodes)
    dc = np.zeros(n_nodes) if want_sens else None
    rep = SimpReport()
    rc = lib().or_simp_solve_nodal(ctypes.byref(desc), np.ascontiguousarray(rho_nodes, np.float64), u,
                                   _ptr(dc), ctypes.byref(rep))
    if rc:
        raise RuntimeError("oracle nodal SIMP solve failed (%d)" % rc)
    return u, dc, rep


def hex8_internal_qp(X, Eq, nu, u, want_K=True):
    """Element force and stiffness with the modulus given per Gauss point."""
    f = np.zeros(24)
    K = np.zeros(576) if want_K else None
    rc = lib().or_hex8_internal_qp(np.ascontiguousarray(X, np.float64), np.ascontiguousarray(Eq, np.float64),
                                   nu, np.ascontiguousarray(u, np.float64), f, _ptr(K))
    if rc:
        raise RuntimeError("non-positive Jacobian")
    return f, (K.reshape(24, 24) if want_K else None)


def simp_load_vector(desc):
    n = (desc.nx + 1) * (desc.ny + 1) * (desc.nz + 1) * 3
    F = np.zeros(n)
    lib().or_simp_load_vector(ctypes.byref(desc), F)
    return F


def simp_fixed_mask(desc):
    n = (desc.nx + 1) * (desc.ny + 1) * (desc.nz + 1) * 3
    fx = np.zeros(n, dtype=np.uint8)
    lib().or_simp_fixed_mask(ctypes.byref(desc), fx)
    return fx


def simp_nodal_modulus(desc, conn, rho_nodes):
    """Moduli and dE/drho at the Gauss points of the elements `conn` (n x 8)."""
    conn = np.ascontiguousarray(conn, np.int32)
    n = conn.shape[0]
    Eq = np.zeros(n * 8)
    dEq = np.zeros(n * 8)
    lib().or_simp_nodal_modulus(ctypes.byref(desc), n, conn.ravel(), np.ascontiguousarray(rho_nodes, np.float64),
                                _ptr(Eq), _ptr(dEq))
    return Eq.reshape(n, 8), dEq.reshape(n, 8)


def simp_modulus(desc, rho):
    rho = np.ascontiguousarray(rho, np.float64)
    E = np.zeros_like(rho)
    dE = np.zeros_like(rho)
    lib().or_simp_modulus(ctypes.byref(desc), rho.shape[0], rho, _ptr(E), _ptr(dE))
    return E, dE


def heat_desc(nx=200, ny=200, k0=1.0, beta=0.01, h=1.0, hc=10.0, Tinf=0.0, rtol=1e-10,
              newton_rtol=1e-10, maxit=100000, max_newton=30, consistent=1, krylov=1):
    return HeatDesc(nx, ny, 1.0, 1.0, k0, beta, h, hc, Tinf, rtol, newton_rtol, maxit,
                    max_newton, consistent, krylov)


def heat_source_field(nx, ny, lo=0.25, hi=0.75, q=1.0):
    """q on elements whose centre lies in [lo,hi]^2 (element-aligned box)."""
    ic = (np.arange(nx) + 0.5) / nx
    jc = (np.arange(ny) + 0.5) / ny
    inside = ((jc[:, None] > lo) & (jc[:, None] < hi)) & ((ic[None, :] > lo) & (ic[None, :] < hi))
    return np.where(inside, q, 0.0).reshape(-1)


def heat_solve(desc, s_elem=None, q_elem=None, want_sens=True):
    n = (desc.nx + 1) * (desc.ny + 1)
    T = np.zeros(n)
    ds = np.zeros(desc.nx * desc.ny) if want_sens else None
    s = None if s_elem is None else np.ascontiguousarray(s_elem, np.float64)
    q = None if q_elem is None else np.ascontiguousarray(q_elem, np.float64)
    rep = HeatReport()
    rc = lib().or_heat_solve(ctypes.byref(desc), _ptr(s), _ptr(q), T, _ptr(ds),
                             ctypes.byref(rep))
    if rc:
        raise RuntimeError("oracle heat solve failed (%d)" % rc)
    return T, ds, rep


def set_threads(n):
    lib().or_set_threads(int(n))


def max_threads():
    return lib().or_max_threads()


def grid_centroids(nx, ny, nz, hx=1.0, hy=1.0, hz=1.0):
    dim = 3 if nz > 0 else 2
    xyz = np.zeros(nx * ny * max(nz, 1) * dim)
    lib().or_grid_centroids(nx, ny, nz, hx, hy, hz, xyz)
    return xyz.reshape(-1, dim)


def filter_points(xyz, radius, x, dv=None, transpose=False):
    """MAST::FilterBase weights over points (O(n^2) search): F x, or F^T x."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n, dim = xyz.shape
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(n)
    dvm = None if dv is None else np.ascontiguousarray(dv, dtype=np.uint8)
    rc = lib().or_filter_points(n, dim, xyz.reshape(-1), radius, _ptr(dvm), x, out, int(transpose))
    if rc:
        raise RuntimeError("oracle filter failed (%d)" % rc)
    return out
