/*
 * mast_oracle.c -- FP64 CPU restatement of MAST's HEX8/QUAD4 hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the FP64 reference the tests compare libmastgpu.so
 * against, and the timed CPU baseline.  The product never links or calls this file.  Each routine cites
 * the reference source it restates (paths relative to the MAST source tree).
 * Parameters, conventions and pinning status are described in mast_oracle.h.
 */
#include "mast_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <sys/time.h>

/* ------------------------------------------------------------------------ */
/* utilities                                                                */
/* ------------------------------------------------------------------------ */
double or_wtime(void) {
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}
int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
void or_free(void *p) { free(p); }

/* 2-point Gauss rule: libMesh QGauss(order 2) for FIRST LAGRANGE
   (src/mesh/fe_base.cpp:103-107, QGauss points/weights are libMesh ext.) */
static const double GP[2] = {-0.57735026918962576451, 0.57735026918962576451};
static const double GW[2] = {1.0, 1.0};

/* libMesh HEX8 / QUAD4 reference node positions (ext.) */
static const double HEX8_N[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                    {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
static const double QUAD4_N[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
/* libMesh QUAD4 side -> local nodes (side 0: y=-1, 1: x=+1, 2: y=+1, 3: x=-1) */
static const int QUAD4_SIDE[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};

/* ------------------------------------------------------------------------ */
/* material matrices                                                        */
/* ------------------------------------------------------------------------ */
/* IsotropicMaterialProperty::StiffnessMatrix3D::operator()
   src/property_cards/isotropic_material_property_card.cpp:512-528 */
void or_iso_stiffness_3d(double E, double nu, double C[36]) {
    memset(C, 0, 36 * sizeof(double));
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            if (i == j)
                C[i * 6 + i] = E * (1. - nu) / (1. - nu - 2. * nu * nu);
            else
                C[i * 6 + j] = E * nu / (1. - nu - 2. * nu * nu);
        }
        C[(i + 3) * 6 + i + 3] = E / 2. / (1. + nu);
    }
}

/* StiffnessMatrix2D::operator() isotropic_material_property_card.cpp:395-426 */
void or_iso_stiffness_2d(double E, double nu, int plane_stress, double C[9]) {
    memset(C, 0, 9 * sizeof(double));
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            if (plane_stress)
                C[i * 3 + j] = (i == j) ? E / (1. - nu * nu) : E * nu / (1. - nu * nu);
            else
                C[i * 3 + j] = (i == j) ? E * (1. - nu) / ((1. + nu) * (1. - 2. * nu))
                                        : E * nu / ((1. + nu) * (1. - 2. * nu));
        }
    C[8] = E / 2. / (1. + nu);
}

/* ------------------------------------------------------------------------ */
/* shape functions and isoparametric maps (libMesh LAGRANGE FIRST, ext.)    */
/* ------------------------------------------------------------------------ */
void or_hex8_shape(const double xi[3], double phi[8], double dphi[24]) {
    for (int a = 0; a < 8; a++) {
        double fx = 0.5 * (1. + HEX8_N[a][0] * xi[0]);
        double fy = 0.5 * (1. + HEX8_N[a][1] * xi[1]);
        double fz = 0.5 * (1. + HEX8_N[a][2] * xi[2]);
        phi[a] = fx * fy * fz;
        dphi[a * 3 + 0] = 0.5 * HEX8_N[a][0] * fy * fz;
        dphi[a * 3 + 1] = 0.5 * HEX8_N[a][1] * fx * fz;
        dphi[a * 3 + 2] = 0.5 * HEX8_N[a][2] * fx * fy;
    }
}

void or_quad4_shape(const double xi[2], double phi[4], double dphi[8]) {
    for (int a = 0; a < 4; a++) {
        double fx = 0.5 * (1. + QUAD4_N[a][0] * xi[0]);
        double fy = 0.5 * (1. + QUAD4_N[a][1] * xi[1]);
        phi[a] = fx * fy;
        dphi[a * 2 + 0] = 0.5 * QUAD4_N[a][0] * fy;
        dphi[a * 2 + 1] = 0.5 * QUAD4_N[a][1] * fx;
    }
}

/* FEBase::init -> libMesh FE reinit: physical gradients and JxW at qp
   (src/mesh/fe_base.cpp:63-130).  X is node-major xyz. Returns det J. */
static double hex8_qp(const double X[24], int qp, double phi[8], double dphi[24],
                      double *JxW) {
    double xi[3] = {GP[qp & 1], GP[(qp >> 1) & 1], GP[(qp >> 2) & 1]};
    double w = GW[qp & 1] * GW[(qp >> 1) & 1] * GW[(qp >> 2) & 1];
    double dref[24];
    or_hex8_shape(xi, phi, dref);
    double J[9] = {0};  /* J[i][j] = d x_j / d xi_i */
    for (int a = 0; a < 8; a++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) J[i * 3 + j] += dref[a * 3 + i] * X[a * 3 + j];
    double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                 J[2] * (J[3] * J[7] - J[4] * J[6]);
    double inv[9];
    inv[0] = (J[4] * J[8] - J[5] * J[7]) / det;
    inv[1] = (J[2] * J[7] - J[1] * J[8]) / det;
    inv[2] = (J[1] * J[5] - J[2] * J[4]) / det;
    inv[3] = (J[5] * J[6] - J[3] * J[8]) / det;
    inv[4] = (J[0] * J[8] - J[2] * J[6]) / det;
    inv[5] = (J[2] * J[3] - J[0] * J[5]) / det;
    inv[6] = (J[3] * J[7] - J[4] * J[6]) / det;
    inv[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    inv[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    /* d phi / d x_j = sum_i (J^{-1})_{j i} d phi / d xi_i */
    for (int a = 0; a < 8; a++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int i = 0; i < 3; i++) s += inv[j * 3 + i] * dref[a * 3 + i];
            dphi[a * 3 + j] = s;
        }
    *JxW = det * w;
    return det;
}

static double quad4_qp(const double X[8], int qp, double phi[4], double dphi[8],
                       double *JxW) {
    double xi[2] = {GP[qp & 1], GP[(qp >> 1) & 1]};
    double w = GW[qp & 1] * GW[(qp >> 1) & 1];
    double dref[8];
    or_quad4_shape(xi, phi, dref);
    double J[4] = {0};
    for (int a = 0; a < 4; a++)
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) J[i * 2 + j] += dref[a * 2 + i] * X[a * 2 + j];
    double det = J[0] * J[3] - J[1] * J[2];
    double inv[4] = {J[3] / det, -J[1] / det, -J[2] / det, J[0] / det};
    for (int a = 0; a < 4; a++)
        for (int j = 0; j < 2; j++)
            dphi[a * 2 + j] = inv[j * 2 + 0] * dref[a * 2 + 0] + inv[j * 2 + 1] * dref[a * 2 + 1];
    *JxW = det * w;
    return det;
}

/* ------------------------------------------------------------------------ */
/* HEX8 linear elasticity                                                   */
/* ------------------------------------------------------------------------ */
/* Strain operator rows (StructuralElement3D::initialize_strain_operator,
   src/elasticity/solid_element_3d.cpp:1272-1304): B is 6 x 24 in
   variable-blocked columns (FEMOperatorMatrix, fem_operator_matrix.h:262-300). */
static void hex8_B(const double dphi[24], double B[144]) {
    memset(B, 0, 144 * sizeof(double));
    for (int a = 0; a < 8; a++) {
        double dx = dphi[a * 3 + 0], dy = dphi[a * 3 + 1], dz = dphi[a * 3 + 2];
        B[0 * 24 + 0 + a] = dx;   /* eps_xx = du/dx */
        B[3 * 24 + 8 + a] = dx;   /* gamma_xy += dv/dx */
        B[5 * 24 + 16 + a] = dx;  /* gamma_zx += dw/dx */
        B[1 * 24 + 8 + a] = dy;   /* eps_yy = dv/dy */
        B[3 * 24 + 0 + a] = dy;   /* gamma_xy += du/dy */
        B[4 * 24 + 16 + a] = dy;  /* gamma_yz += dw/dy */
        B[2 * 24 + 16 + a] = dz;  /* eps_zz = dw/dz */
        B[4 * 24 + 8 + a] = dz;   /* gamma_yz += dv/dz */
        B[5 * 24 + 0 + a] = dz;   /* gamma_zx += du/dz */
    }
}

/* StructuralElement3D::internal_residual, linear-strain branch
   (solid_element_3d.cpp:135-423): per qp eps = B u, sigma = C eps,
   f += JxW B^T sigma (:296-297), K += JxW B^T C B (:327-329).  Only the
   translational 24x24 block is returned (rotational dofs are decoupled and
   regularised at :415-417). */
/* Eq non-NULL: the modulus at each quadrature point (a MeshFieldFunction
   density interpolated there, example_6.cpp:104-137), else E throughout */
static int hex8_internal_impl(const double X[24], double E, const double *Eq, double nu,
                              const double u[24], double f[24], double K[576]) {
    double C[36], phi[8], dphi[24], B[144], JxW;
    or_iso_stiffness_3d(E, nu, C);
    memset(f, 0, 24 * sizeof(double));
    if (K) memset(K, 0, 576 * sizeof(double));
    for (int qp = 0; qp < 8; qp++) {
        if (Eq) or_iso_stiffness_3d(Eq[qp], nu, C);
        if (hex8_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        hex8_B(dphi, B);
        double eps[6] = {0}, sig[6] = {0};
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 24; c++) eps[r] += B[r * 24 + c] * u[c];
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++) sig[r] += C[r * 6 + c] * eps[c];
        for (int c = 0; c < 24; c++) {
            double s = 0;
            for (int r = 0; r < 6; r++) s += B[r * 24 + c] * sig[r];
            f[c] += JxW * s;
        }
        if (K) {
            double CB[144];
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 24; c++) {
                    double s = 0;
                    for (int k = 0; k < 6; k++) s += C[r * 6 + k] * B[k * 24 + c];
                    CB[r * 24 + c] = s;
                }
            for (int i = 0; i < 24; i++)
                for (int j = 0; j < 24; j++) {
                    double s = 0;
                    for (int r = 0; r < 6; r++) s += B[r * 24 + i] * CB[r * 24 + j];
                    K[i * 24 + j] += JxW * s;
                }
        }
    }
    return 0;
}

int or_hex8_internal(const double X[24], double E, double nu, const double u[24],
                     double f[24], double K[576]) {
    return hex8_internal_impl(X, E, NULL, nu, u, f, K);
}

int or_hex8_internal_qp(const double X[24], const double Eq[8], double nu, const double u[24],
                        double f[24], double K[576]) {
    return hex8_internal_impl(X, 0.0, Eq, nu, u, f, K);
}

/* StructuralElement3D::internal_residual, nonlinear-strain branch
   (solid_element_3d.cpp:299-409 with initialize_green_lagrange_strain_operator
   :1309-1463): total Lagrangian, F = grad u at the reference configuration,
   Green-Lagrange strain E = (F + F^T + F^T F) / 2 in Voigt order with
   engineering shears, S = C E; f += JxW B_L^T S with B_L = B_lin + the
   displacement-dependent rows (the reference's mat_x/y/z times Bmat_nl_x/y/z),
   K += JxW (B_L^T C B_L + the geometric stiffness grad N_a . S . grad N_b per
   component, the reference's Bmat_nl_u/v/w products with the stress tensor).
   The incompatible-mode and rotational-dof terms are absent as in the linear
   branch. */
int or_hex8_internal_gl(const double X[24], double E, double nu, const double u[24],
                        double f[24], double K[576]) {
    double C[36], phi[8], dphi[24], JxW;
    or_iso_stiffness_3d(E, nu, C);
    memset(f, 0, 24 * sizeof(double));
    if (K) memset(K, 0, 576 * sizeof(double));
    static const int VJ[6] = {0, 1, 2, 0, 1, 0}, VK[6] = {0, 1, 2, 1, 2, 2};
    for (int qp = 0; qp < 8; qp++) {
        if (hex8_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        double F[9] = {0};  /* F[i][j] = d u_i / d X_j */
        for (int i = 0; i < 3; i++)
            for (int a = 0; a < 8; a++)
                for (int j = 0; j < 3; j++) F[i * 3 + j] += u[i * 8 + a] * dphi[a * 3 + j];
        double eps[6], sig[6] = {0}, BL[144];
        for (int r = 0; r < 6; r++) {
            const int j = VJ[r], k = VK[r];
            double e = 0.5 * (F[j * 3 + k] + F[k * 3 + j]);
            for (int m = 0; m < 3; m++) e += 0.5 * F[m * 3 + j] * F[m * 3 + k];
            eps[r] = (r < 3) ? e : 2.0 * e;
        }
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++) sig[r] += C[r * 6 + c] * eps[c];
        /* B_L: the strain variation of dof (component i, node a), dF_mn = delta_im g_n:
           dE_jk = (delta_ij g_k + delta_ik g_j + g_j F_ik + F_ij g_k) / 2 */
        for (int i = 0; i < 3; i++)
            for (int a = 0; a < 8; a++) {
                const double *g = dphi + a * 3;
                for (int r = 0; r < 6; r++) {
                    const int j = VJ[r], k = VK[r];
                    double de = 0.5 * ((i == j ? g[k] : 0.0) + (i == k ? g[j] : 0.0) + g[j] * F[i * 3 + k] +
                                       F[i * 3 + j] * g[k]);
                    BL[r * 24 + i * 8 + a] = (r < 3) ? de : 2.0 * de;
                }
            }
        for (int c = 0; c < 24; c++) {
            double s = 0;
            for (int r = 0; r < 6; r++) s += BL[r * 24 + c] * sig[r];
            f[c] += JxW * s;
        }
        if (K) {
            const double St[9] = {sig[0], sig[3], sig[5], sig[3], sig[1], sig[4], sig[5], sig[4], sig[2]};
            double CB[144];
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 24; c++) {
                    double s = 0;
                    for (int q = 0; q < 6; q++) s += C[r * 6 + q] * BL[q * 24 + c];
                    CB[r * 24 + c] = s;
                }
            for (int i = 0; i < 24; i++)
                for (int j = 0; j < 24; j++) {
                    double s = 0;
                    for (int r = 0; r < 6; r++) s += BL[r * 24 + i] * CB[r * 24 + j];
                    K[i * 24 + j] += JxW * s;
                }
            for (int a = 0; a < 8; a++)
                for (int b = 0; b < 8; b++) {
                    double gsg = 0;
                    for (int m = 0; m < 3; m++)
                        for (int n = 0; n < 3; n++) gsg += dphi[a * 3 + m] * St[m * 3 + n] * dphi[b * 3 + n];
                    for (int i = 0; i < 3; i++) K[(i * 8 + a) * 24 + i * 8 + b] += JxW * gsg;
                }
        }
    }
    return 0;
}

/* StructuralElement3D::internal_residual_sensitivity, linear branch
   (solid_element_3d.cpp:567-788): C replaced by dC/dp (:640).  With only E
   depending on p (StiffnessMatrix3D::derivative,
   isotropic_material_property_card.cpp:533-567, dnu/dp = 0) dC/dp = dE C(1,nu). */
/* StructuralElement3D::calculate_stress (solid_element_3d.cpp:1147-1270): per
   Gauss point the strain of initialize_green_lagrange_strain_operator (B u for
   the linear strain, (H + H^T + H^T H)/2 in Voigt form with engineering shears
   for NONLINEAR_STRAIN), stress C eps, its derivative d sigma / d u = C B (C B_L
   for the nonlinear strain, nullable) and JxW; von Mises per point by
   StressStrainOutputBase::Data::von_Mises_stress (stress_output_base.cpp:183-195).
   sig[qp*6 + r], dsig[(qp*6 + r)*24 + c] with var-blocked dofs c = i 8 + a. */
int or_hex8_stress(const double X[24], double E, double nu, const double u[24], int nonlinear,
                   double sig[48], double vm[8], double JxW_out[8], double *dsig) {
    double C[36], phi[8], dphi[24], JxW;
    or_iso_stiffness_3d(E, nu, C);
    static const int VJ[6] = {0, 1, 2, 0, 1, 0}, VK[6] = {0, 1, 2, 1, 2, 2};
    for (int qp = 0; qp < 8; qp++) {
        if (hex8_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        JxW_out[qp] = JxW;
        double F[9] = {0}, eps[6], B[144];
        for (int i = 0; i < 3; i++)
            for (int a = 0; a < 8; a++)
                for (int j = 0; j < 3; j++) F[i * 3 + j] += u[i * 8 + a] * dphi[a * 3 + j];
        if (!nonlinear) {
            hex8_B(dphi, B);
            for (int r = 0; r < 6; r++) {
                double e = 0;
                for (int c = 0; c < 24; c++) e += B[r * 24 + c] * u[c];
                eps[r] = e;
            }
        } else {
            for (int r = 0; r < 6; r++) {
                const int j = VJ[r], k = VK[r];
                double e = 0.5 * (F[j * 3 + k] + F[k * 3 + j]);
                for (int m = 0; m < 3; m++) e += 0.5 * F[m * 3 + j] * F[m * 3 + k];
                eps[r] = (r < 3) ? e : 2.0 * e;
            }
            for (int i = 0; i < 3; i++)
                for (int a = 0; a < 8; a++) {
                    const double *g = dphi + a * 3;
                    for (int r = 0; r < 6; r++) {
                        const int j = VJ[r], k = VK[r];
                        double de = 0.5 * ((i == j ? g[k] : 0.0) + (i == k ? g[j] : 0.0) +
                                           g[j] * F[i * 3 + k] + F[i * 3 + j] * g[k]);
                        B[r * 24 + i * 8 + a] = (r < 3) ? de : 2.0 * de;
                    }
                }
        }
        double *s = sig + qp * 6;
        for (int r = 0; r < 6; r++) {
            double v = 0;
            for (int c = 0; c < 6; c++) v += C[r * 6 + c] * eps[c];
            s[r] = v;
        }
        vm[qp] = sqrt(0.5 * ((s[0] - s[1]) * (s[0] - s[1]) + (s[1] - s[2]) * (s[1] - s[2]) +
                             (s[2] - s[0]) * (s[2] - s[0])) +
                      3.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]));
        if (dsig)
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 24; c++) {
                    double v = 0;
                    for (int q = 0; q < 6; q++) v += C[r * 6 + q] * B[q * 24 + c];
                    dsig[(qp * 6 + r) * 24 + c] = v;
                }
    }
    return 0;
}

int or_hex8_internal_sens(const double X[24], double dE, double nu,
                          const double u[24], double df[24]) {
    return or_hex8_internal(X, dE, nu, u, df, NULL);
}

/* ------------------------------------------------------------------------ */
/* QUAD4 membrane (StructuralElement2D, linear strain, NO_BENDING)          */
/* ------------------------------------------------------------------------ */
/* structural_element_2d.cpp:1076-1227 with _internal_residual_operation
   :1766-1890 (membrane terms): A = plane-stress C * h
   (isotropic_material_property_card.cpp:395-426 times the section thickness);
   B_lin rows [du/dx ; dv/dy ; du/dy + dv/dx] over the (u, v) blocks. */
int or_quad4_membrane_internal(const double X[8], double E, double nu, double h,
                               const double u[8], double f[8], double K[64]) {
    double C[9], phi[4], dphi[8], JxW;
    or_iso_stiffness_2d(E, nu, 1, C);
    for (int i = 0; i < 9; i++) C[i] *= h;
    memset(f, 0, 8 * sizeof(double));
    if (K) memset(K, 0, 64 * sizeof(double));
    for (int qp = 0; qp < 4; qp++) {
        if (quad4_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        double B[24];
        memset(B, 0, sizeof(B));
        for (int a = 0; a < 4; a++) {
            B[0 * 8 + a] = dphi[a * 2 + 0];
            B[1 * 8 + 4 + a] = dphi[a * 2 + 1];
            B[2 * 8 + a] = dphi[a * 2 + 1];
            B[2 * 8 + 4 + a] = dphi[a * 2 + 0];
        }
        double eps[3] = {0}, sig[3] = {0};
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 8; c++) eps[r] += B[r * 8 + c] * u[c];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) sig[r] += C[r * 3 + c] * eps[c];
        for (int c = 0; c < 8; c++) {
            double s = 0;
            for (int r = 0; r < 3; r++) s += B[r * 8 + c] * sig[r];
            f[c] += JxW * s;
        }
        if (K)
            for (int i = 0; i < 8; i++)
                for (int j = 0; j < 8; j++) {
                    double s = 0;
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 3; c++) s += B[r * 8 + i] * C[r * 3 + c] * B[c * 8 + j];
                    K[i * 8 + j] += JxW * s;
                }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* QUAD4 conduction                                                         */
/* ------------------------------------------------------------------------ */
/* HeatConductionElementBase::internal_residual
   (src/heat_conduction/heat_conduction_elem_base.cpp:53-149).
   Conductance k_ij = k(T_qp) delta_ij h (isotropic_material_property_card.cpp:
   716-732 times solid_2d_section_element_property_card.cpp:940-954) with
   k(T) = k0 (1 + beta T) s.  f += JxW dB_i^T q_i, q_i = k_ij dT/dx_j (:94-107);
   K += JxW k_ij dB_i^T dB_j (:112-120); if consistent, the temperature
   derivative term JxW dT/dx_j dk_ij/dT dB_i^T B of :125-142. */
int or_quad4_heat_internal(const double X[8], double k0, double beta, double s,
                           double h, const double T[4], int consistent,
                           double f[4], double K[16]) {
    double phi[4], dphi[8], JxW;
    memset(f, 0, 4 * sizeof(double));
    if (K) memset(K, 0, 16 * sizeof(double));
    for (int qp = 0; qp < 4; qp++) {
        if (quad4_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        double Tq = 0, g[2] = {0, 0};
        for (int a = 0; a < 4; a++) {
            Tq += phi[a] * T[a];
            g[0] += dphi[a * 2 + 0] * T[a];
            g[1] += dphi[a * 2 + 1] * T[a];
        }
        double k = k0 * (1. + beta * Tq) * s * h;
        double dk = k0 * beta * s * h;
        for (int a = 0; a < 4; a++)
            f[a] += JxW * (dphi[a * 2 + 0] * k * g[0] + dphi[a * 2 + 1] * k * g[1]);
        if (K)
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) {
                    double v = k * (dphi[a * 2] * dphi[b * 2] + dphi[a * 2 + 1] * dphi[b * 2 + 1]);
                    if (consistent)
                        v += (dphi[a * 2] * g[0] + dphi[a * 2 + 1] * g[1]) * dk * phi[b];
                    K[a * 4 + b] += JxW * v;
                }
    }
    return 0;
}

/* internal_residual_sensitivity (heat_conduction_elem_base.cpp:553-617):
   the conductance replaced by its parameter derivative dk/dp = (a + b T_qp) h. */
int or_quad4_heat_internal_sens(const double X[8], double a, double b, double h,
                                const double T[4], double df[4]) {
    double phi[4], dphi[8], JxW;
    memset(df, 0, 4 * sizeof(double));
    for (int qp = 0; qp < 4; qp++) {
        if (quad4_qp(X, qp, phi, dphi, &JxW) <= 0.) return -1;
        double Tq = 0, g[2] = {0, 0};
        for (int n = 0; n < 4; n++) {
            Tq += phi[n] * T[n];
            g[0] += dphi[n * 2 + 0] * T[n];
            g[1] += dphi[n * 2 + 1] * T[n];
        }
        double dk = (a + b * Tq) * h;
        for (int n = 0; n < 4; n++)
            df[n] += JxW * dk * (dphi[n * 2] * g[0] + dphi[n * 2 + 1] * g[1]);
    }
    return 0;
}

/* surface_convection_residual (heat_conduction_elem_base.cpp:1100-1154):
   2-point side rule (fe_base.cpp:164-167), f += JxW phi th h (T - Tinf),
   K += JxW phi phi^T th h. */
void or_quad4_heat_convection(const double X[8], int side, double hc, double Tinf,
                              double th, const double T[4], double f[4], double K[16]) {
    int n0 = QUAD4_SIDE[side][0], n1 = QUAD4_SIDE[side][1];
    double dx = X[n1 * 2] - X[n0 * 2], dy = X[n1 * 2 + 1] - X[n0 * 2 + 1];
    double L = sqrt(dx * dx + dy * dy);
    memset(f, 0, 4 * sizeof(double));
    if (K) memset(K, 0, 16 * sizeof(double));
    for (int qp = 0; qp < 2; qp++) {
        double t = GP[qp];
        double JxW = GW[qp] * 0.5 * L;
        double phi[4] = {0, 0, 0, 0};
        phi[n0] = 0.5 * (1. - t);
        phi[n1] = 0.5 * (1. + t);
        double Tq = 0;
        for (int a = 0; a < 4; a++) Tq += phi[a] * T[a];
        for (int a = 0; a < 4; a++) f[a] += JxW * phi[a] * th * hc * (Tq - Tinf);
        if (K)
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) K[a * 4 + b] += JxW * phi[a] * phi[b] * th * hc;
    }
}

/* surface_flux_residual (heat_conduction_elem_base.cpp:876-913): the residual
   gets f += JxW phi q_n th over the edge (2-point rule), q_n the outward flux. */
void or_quad4_heat_flux(const double X[8], int side, double flux, double th, double f[4]) {
    int n0 = QUAD4_SIDE[side][0], n1 = QUAD4_SIDE[side][1];
    double dx = X[n1 * 2] - X[n0 * 2], dy = X[n1 * 2 + 1] - X[n0 * 2 + 1];
    double L = sqrt(dx * dx + dy * dy);
    memset(f, 0, 4 * sizeof(double));
    for (int qp = 0; qp < 2; qp++) {
        double t = GP[qp], JxW = GW[qp] * 0.5 * L;
        f[n0] += JxW * 0.5 * (1. - t) * flux * th;
        f[n1] += JxW * 0.5 * (1. + t) * flux * th;
    }
}

/* libMesh Hex8 side -> node map (counter-clockwise seen from outside) */
static const int HEX8_SIDE[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                    {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

/* StructuralElement3D::surface_pressure_residual (solid_element_3d.cpp:815-876)
   on the side's own QUAD4 finite element: per 2x2 Gauss point JxW = |x_xi x
   x_eta|, unit outward normal n = (x_xi x x_eta)/JxW, and the residual gets
   -JxW phi p n; returned here as the external load f_ext[d*8 + a] (var-blocked)
   = +sum_qp JxW phi_a p n_d. */
void or_hex8_pressure(const double X[24], int side, double p, double f[24]) {
    memset(f, 0, 24 * sizeof(double));
    for (int qp = 0; qp < 4; qp++) {
        double xi[2] = {GP[qp & 1], GP[qp >> 1]}, phi[4], dphi[8];
        or_quad4_shape(xi, phi, dphi);
        double t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
        for (int i = 0; i < 4; i++) {
            const double *x = X + 3 * HEX8_SIDE[side][i];
            for (int d = 0; d < 3; d++) {
                t1[d] += dphi[i * 2] * x[d];
                t2[d] += dphi[i * 2 + 1] * x[d];
            }
        }
        double c[3] = {t1[1] * t2[2] - t1[2] * t2[1], t1[2] * t2[0] - t1[0] * t2[2],
                       t1[0] * t2[1] - t1[1] * t2[0]};
        const double area = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const double JxW = GW[qp & 1] * GW[qp >> 1] * area;
        for (int i = 0; i < 4; i++)
            for (int d = 0; d < 3; d++) f[d * 8 + HEX8_SIDE[side][i]] += JxW * phi[i] * p * (c[d] / area);
    }
}

/* volume_heat_source_residual (heat_conduction_elem_base.cpp:1710-1745):
   f -= JxW phi q th. */
void or_quad4_heat_source(const double X[8], double q, double th, double f[4]) {
    double phi[4], dphi[8], JxW;
    memset(f, 0, 4 * sizeof(double));
    for (int qp = 0; qp < 4; qp++) {
        quad4_qp(X, qp, phi, dphi, &JxW);
        for (int a = 0; a < 4; a++) f[a] -= JxW * phi[a] * q * th;
    }
}

/* ------------------------------------------------------------------------ */
/* structured meshes                                                        */
/* ------------------------------------------------------------------------ */
/* libMesh MeshTools::Generation::build_cube / build_square numbering (ext.):
   node (i,j,k) = i + (nx+1)(j + (ny+1)k); element x-fastest. */
void or_grid_hex8(int nx, int ny, int nz, double lx, double ly, double lz,
                  double *coords, int32_t *conn) {
    int64_t NX = nx + 1, NY = ny + 1;
    for (int k = 0; k <= nz; k++)
        for (int j = 0; j <= ny; j++)
            for (int i = 0; i <= nx; i++) {
                int64_t n = i + NX * (j + NY * k);
                coords[n * 3 + 0] = lx * i / nx;
                coords[n * 3 + 1] = ly * j / ny;
                coords[n * 3 + 2] = lz * k / nz;
            }
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int64_t e = i + (int64_t)nx * (j + (int64_t)ny * k);
                int64_t n0 = i + NX * (j + NY * k);
                int32_t *c = conn + e * 8;
                c[0] = (int32_t)n0;
                c[1] = (int32_t)(n0 + 1);
                c[2] = (int32_t)(n0 + 1 + NX);
                c[3] = (int32_t)(n0 + NX);
                c[4] = (int32_t)(n0 + NX * NY);
                c[5] = (int32_t)(n0 + 1 + NX * NY);
                c[6] = (int32_t)(n0 + 1 + NX + NX * NY);
                c[7] = (int32_t)(n0 + NX + NX * NY);
            }
}

void or_grid_quad4(int nx, int ny, double lx, double ly, double *coords, int32_t *conn) {
    int64_t NX = nx + 1;
    for (int j = 0; j <= ny; j++)
        for (int i = 0; i <= nx; i++) {
            int64_t n = i + NX * j;
            coords[n * 2 + 0] = lx * i / nx;
            coords[n * 2 + 1] = ly * j / ny;
        }
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int64_t e = i + (int64_t)nx * j, n0 = i + NX * j;
            conn[e * 4 + 0] = (int32_t)n0;
            conn[e * 4 + 1] = (int32_t)(n0 + 1);
            conn[e * 4 + 2] = (int32_t)(n0 + 1 + NX);
            conn[e * 4 + 3] = (int32_t)(n0 + NX);
        }
}

/* ------------------------------------------------------------------------ */
/* sparse pattern, colouring, SpMV                                          */
/* ------------------------------------------------------------------------ */
static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* node adjacency through shared elements (the pattern libMesh's DofMap
   builds for the system matrix, ext.) */
static int64_t node_adjacency(int npe, int64_t n_nodes, int64_t n_elems,
                              const int32_t *conn, int32_t **adj_ptr_out,
                              int32_t **adj_out) {
    int64_t *cnt = (int64_t *)calloc((size_t)n_nodes + 1, sizeof(int64_t));
    for (int64_t e = 0; e < n_elems; e++)
        for (int a = 0; a < npe; a++) cnt[conn[e * npe + a] + 1] += npe;
    for (int64_t n = 0; n < n_nodes; n++) cnt[n + 1] += cnt[n];
    int32_t *tmp = (int32_t *)malloc((size_t)cnt[n_nodes] * sizeof(int32_t));
    int64_t *fill = (int64_t *)calloc((size_t)n_nodes, sizeof(int64_t));
    for (int64_t e = 0; e < n_elems; e++)
        for (int a = 0; a < npe; a++) {
            int32_t na = conn[e * npe + a];
            for (int b = 0; b < npe; b++) tmp[cnt[na] + fill[na]++] = conn[e * npe + b];
        }
    int32_t *aptr = (int32_t *)malloc(((size_t)n_nodes + 1) * sizeof(int32_t));
    int64_t total = 0;
    aptr[0] = 0;
    for (int64_t n = 0; n < n_nodes; n++) {
        int32_t *seg = tmp + cnt[n];
        int64_t m = cnt[n + 1] - cnt[n], u = 0;
        qsort(seg, (size_t)m, sizeof(int32_t), cmp_i32);
        for (int64_t i = 0; i < m; i++)
            if (i == 0 || seg[i] != seg[i - 1]) seg[u++] = seg[i];
        fill[n] = u;
        total += u;
        aptr[n + 1] = (int32_t)total;
    }
    int32_t *adj = (int32_t *)malloc((size_t)total * sizeof(int32_t));
    for (int64_t n = 0; n < n_nodes; n++)
        memcpy(adj + aptr[n], tmp + cnt[n], (size_t)fill[n] * sizeof(int32_t));
    free(tmp);
    free(fill);
    free(cnt);
    *adj_ptr_out = aptr;
    *adj_out = adj;
    return total;
}

int64_t or_csr_pattern(int npe, int dpn, int64_t n_nodes, int64_t n_elems,
                       const int32_t *conn, int32_t *rowptr, int32_t *cols) {
    int32_t *aptr, *adj;
    node_adjacency(npe, n_nodes, n_elems, conn, &aptr, &adj);
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int64_t n = 0; n < n_nodes; n++) {
        int64_t deg = aptr[n + 1] - aptr[n];
        for (int c = 0; c < dpn; c++) {
            if (cols)
                for (int64_t k = 0; k < deg; k++)
                    for (int d = 0; d < dpn; d++)
                        cols[nnz + k * dpn + d] = adj[aptr[n] + k] * dpn + d;
            nnz += deg * dpn;
            rowptr[n * dpn + c + 1] = (int32_t)nnz;
        }
    }
    free(aptr);
    free(adj);
    return nnz;
}

/* greedy element colouring: no two elements of one colour share a node */
int or_color_elements(int npe, int64_t n_nodes, int64_t n_elems, const int32_t *conn,
                      int32_t *color) {
    uint64_t *used = (uint64_t *)calloc((size_t)n_nodes, sizeof(uint64_t));
    int ncol = 0;
    for (int64_t e = 0; e < n_elems; e++) {
        uint64_t m = 0;
        for (int a = 0; a < npe; a++) m |= used[conn[e * npe + a]];
        int c = 0;
        while (c < 64 && (m >> c) & 1ull) c++;
        color[e] = c;
        if (c + 1 > ncol) ncol = c + 1;
        for (int a = 0; a < npe; a++) used[conn[e * npe + a]] |= 1ull << c;
    }
    free(used);
    return ncol;
}

void or_csr_spmv(int64_t n, const int32_t *rowptr, const int32_t *cols,
                 const double *vals, const double *x, double *y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double s = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) s += vals[k] * x[cols[k]];
        y[i] = s;
    }
}

void or_csr_transpose(int64_t n, const int32_t *rowptr, const int32_t *cols,
                      const double *vals, int32_t *rowptr_t, int32_t *cols_t,
                      double *vals_t) {
    int64_t nnz = rowptr[n];
    int32_t *fill = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    memset(rowptr_t, 0, ((size_t)n + 1) * sizeof(int32_t));
    for (int64_t k = 0; k < nnz; k++) rowptr_t[cols[k] + 1]++;
    for (int64_t i = 0; i < n; i++) rowptr_t[i + 1] += rowptr_t[i];
    for (int64_t i = 0; i < n; i++)
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            int32_t c = cols[k];
            int32_t p = rowptr_t[c] + fill[c]++;
            cols_t[p] = (int32_t)i;
            vals_t[p] = vals[k];
        }
    free(fill);
}

/* position of column c in row r (binary search; rows are sorted) */
static int64_t csr_find(const int32_t *rowptr, const int32_t *cols, int64_t r, int32_t c) {
    int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) / 2;
        if (cols[mid] == c) return mid;
        if (cols[mid] < c)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

/* Dirichlet constraint by elimination: fixed rows and columns zeroed, unit
   diagonal (libMesh constrain_element_matrix_and_vector is ext.; the free-dof
   block is identical under either convention). */
static void apply_fixed(int64_t n, const int32_t *rowptr, const int32_t *cols,
                        double *vals, const uint8_t *fixed) {
    if (!fixed) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++)
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            int32_t c = cols[k];
            if (fixed[i] || fixed[c]) vals[k] = (c == i) ? 1.0 : 0.0;
        }
}

/* NonlinearImplicitAssembly::residual_and_jacobian element loop
   (src/base/nonlinear_implicit_assembly.cpp:111-186): gather, element
   calculation, scatter add into the global matrix.  Colours make the
   parallel scatter race-free. */
static int assemble_hex8_impl(int64_t n_nodes, int64_t n_elems, const double *coords,
                              const int32_t *conn, const double *E_elem, const double *E_qp,
                              double nu, const int32_t *rowptr, const int32_t *cols, double *vals,
                              const uint8_t *fixed, int n_colors, const int32_t *color) {
    int64_t n = n_nodes * 3;
    memset(vals, 0, (size_t)rowptr[n] * sizeof(double));
    int bad = 0;
    for (int c = 0; c < n_colors; c++) {
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
        for (int64_t e = 0; e < n_elems; e++) {
            if (color && color[e] != c) continue;
            if (!color && c > 0) continue;
            const int32_t *en = conn + e * 8;
            double X[24], u0[24] = {0}, f[24], K[576];
            for (int a = 0; a < 8; a++)
                for (int d = 0; d < 3; d++) X[a * 3 + d] = coords[(int64_t)en[a] * 3 + d];
            if (E_qp ? or_hex8_internal_qp(X, E_qp + e * 8, nu, u0, f, K)
                     : or_hex8_internal(X, E_elem[e], nu, u0, f, K))
                bad |= 1;
            for (int a = 0; a < 8; a++)
                for (int i = 0; i < 3; i++) {
                    int64_t row = (int64_t)en[a] * 3 + i;
                    for (int b = 0; b < 8; b++) {
                        int64_t p = csr_find(rowptr, cols, row, en[b] * 3);
                        for (int j = 0; j < 3; j++)
                            vals[p + j] += K[(i * 8 + a) * 24 + j * 8 + b];
                    }
                }
        }
    }
    apply_fixed(n, rowptr, cols, vals, fixed);
    return bad ? -1 : 0;
}

int or_assemble_hex8(int64_t n_nodes, int64_t n_elems, const double *coords,
                     const int32_t *conn, const double *E_elem, double nu,
                     const int32_t *rowptr, const int32_t *cols, double *vals,
                     const uint8_t *fixed, int n_colors, const int32_t *color) {
    return assemble_hex8_impl(n_nodes, n_elems, coords, conn, E_elem, NULL, nu, rowptr, cols, vals,
                              fixed, n_colors, color);
}

int or_assemble_hex8_qp(int64_t n_nodes, int64_t n_elems, const double *coords,
                        const int32_t *conn, const double *E_qp, double nu,
                        const int32_t *rowptr, const int32_t *cols, double *vals,
                        const uint8_t *fixed, int n_colors, const int32_t *color) {
    return assemble_hex8_impl(n_nodes, n_elems, coords, conn, NULL, E_qp, nu, rowptr, cols, vals,
                              fixed, n_colors, color);
}

int or_assemble_quad4_membrane(int64_t n_nodes, int64_t n_elems, const double *coords,
                               const int32_t *conn, const double *E_elem, double nu,
                               double h, const int32_t *rowptr, const int32_t *cols,
                               double *vals, const uint8_t *fixed) {
    int64_t n = n_nodes * 2;
    memset(vals, 0, (size_t)rowptr[n] * sizeof(double));
    for (int64_t e = 0; e < n_elems; e++) {
        const int32_t *en = conn + e * 4;
        double X[8], u0[8] = {0}, f[8], K[64];
        for (int a = 0; a < 4; a++)
            for (int d = 0; d < 2; d++) X[a * 2 + d] = coords[(int64_t)en[a] * 2 + d];
        if (or_quad4_membrane_internal(X, E_elem[e], nu, h, u0, f, K)) return -1;
        for (int a = 0; a < 4; a++)
            for (int i = 0; i < 2; i++) {
                int64_t row = (int64_t)en[a] * 2 + i;
                for (int b = 0; b < 4; b++) {
                    int64_t p = csr_find(rowptr, cols, row, en[b] * 2);
                    for (int j = 0; j < 2; j++) vals[p + j] += K[(i * 4 + a) * 8 + j * 4 + b];
                }
            }
    }
    apply_fixed(n, rowptr, cols, vals, fixed);
    return 0;
}

/* HeatConductionNonlinearAssemblyElemOperations::elem_calculations
   (src/heat_conduction/heat_conduction_nonlinear_assembly.cpp:81-98):
   internal + side convection + volume source, summed into R and J. */
int or_assemble_quad4_heat(int64_t n_nodes, int64_t n_elems, const double *coords,
                           const int32_t *conn, double k0, double beta,
                           const double *s_elem, double h, const double *q_elem,
                           int64_t n_conv, const int32_t *conv_elem,
                           const int32_t *conv_side, double hc, double Tinf,
                           const double *T, int consistent,
                           const int32_t *rowptr, const int32_t *cols, double *vals,
                           double *R, const uint8_t *fixed) {
    int64_t n = n_nodes;
    if (vals) memset(vals, 0, (size_t)rowptr[n] * sizeof(double));
    if (R) memset(R, 0, (size_t)n * sizeof(double));
    for (int64_t e = 0; e < n_elems; e++) {
        const int32_t *en = conn + e * 4;
        double X[8], Te[4], f[4], K[16], fs[4];
        for (int a = 0; a < 4; a++) {
            X[a * 2] = coords[(int64_t)en[a] * 2];
            X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
            Te[a] = T[en[a]];
        }
        if (or_quad4_heat_internal(X, k0, beta, s_elem ? s_elem[e] : 1.0, h, Te, consistent,
                                   f, vals ? K : NULL))
            return -1;
        if (q_elem && q_elem[e] != 0.0) {
            or_quad4_heat_source(X, q_elem[e], h, fs);
            for (int a = 0; a < 4; a++) f[a] += fs[a];
        }
        for (int a = 0; a < 4; a++) {
            if (R) R[en[a]] += f[a];
            if (vals)
                for (int b = 0; b < 4; b++) {
                    int64_t p = csr_find(rowptr, cols, en[a], en[b]);
                    vals[p] += K[a * 4 + b];
                }
        }
    }
    for (int64_t s = 0; s < n_conv; s++) {
        int64_t e = conv_elem[s];
        const int32_t *en = conn + e * 4;
        double X[8], Te[4], f[4], K[16];
        for (int a = 0; a < 4; a++) {
            X[a * 2] = coords[(int64_t)en[a] * 2];
            X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
            Te[a] = T[en[a]];
        }
        or_quad4_heat_convection(X, conv_side[s], hc, Tinf, h, Te, f, K);
        for (int a = 0; a < 4; a++) {
            if (R) R[en[a]] += f[a];
            if (vals)
                for (int b = 0; b < 4; b++) {
                    int64_t p = csr_find(rowptr, cols, en[a], en[b]);
                    vals[p] += K[a * 4 + b];
                }
        }
    }
    if (fixed) {
        if (R)
            for (int64_t i = 0; i < n; i++)
                if (fixed[i]) R[i] = T[i];
        if (vals) apply_fixed(n, rowptr, cols, vals, fixed);
    }
    return 0;
}

/* NonlinearImplicitAssembly::residual_and_jacobian
   (src/base/nonlinear_implicit_assembly.cpp:111-186) over the Green-Lagrange
   HEX8 element: R = f_int(u) - F with node-interleaved global dofs (3 node + c),
   tangent scattered into the CSR; constrained rows R_d = u_d, rows and columns
   eliminated with a unit diagonal. */
int or_assemble_hex8_gl(int64_t n_nodes, int64_t n_elems, const double *coords,
                        const int32_t *conn, const double *E_elem, double nu, const double *u,
                        const double *F, const int32_t *rowptr, const int32_t *cols,
                        double *vals, double *R, const uint8_t *fixed) {
    int64_t n = n_nodes * 3;
    if (vals) memset(vals, 0, (size_t)rowptr[n] * sizeof(double));
    if (R) memset(R, 0, (size_t)n * sizeof(double));
    for (int64_t e = 0; e < n_elems; e++) {
        const int32_t *en = conn + e * 8;
        double X[24], ue[24], f[24], K[576];
        for (int a = 0; a < 8; a++)
            for (int d = 0; d < 3; d++) {
                X[a * 3 + d] = coords[(int64_t)en[a] * 3 + d];
                ue[d * 8 + a] = u[(int64_t)en[a] * 3 + d];
            }
        if (or_hex8_internal_gl(X, E_elem[e], nu, ue, f, vals ? K : NULL)) return -1;
        for (int a = 0; a < 8; a++)
            for (int i = 0; i < 3; i++) {
                int64_t row = (int64_t)en[a] * 3 + i;
                if (R) R[row] += f[i * 8 + a];
                if (vals)
                    for (int b = 0; b < 8; b++) {
                        int64_t p = csr_find(rowptr, cols, row, en[b] * 3);
                        for (int j = 0; j < 3; j++) vals[p + j] += K[(i * 8 + a) * 24 + j * 8 + b];
                    }
            }
    }
    if (R)
        for (int64_t i = 0; i < n; i++) {
            if (F) R[i] -= F[i];
            if (fixed && fixed[i]) R[i] = u[i];
        }
    if (vals) apply_fixed(n, rowptr, cols, vals, fixed);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Krylov solvers (the role PETSc KSP plays under SNES, ext.)               */
/* ------------------------------------------------------------------------ */
static double dot(int64_t n, const double *a, const double *b) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static void jacobi_diag(int64_t n, const int32_t *rowptr, const int32_t *cols,
                        const double *vals, double *dinv) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double d = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
            if (cols[k] == i) d = vals[k];
        dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
    }
}

/* Jacobi-preconditioned CG; stops on ||b - A x||_2 <= rtol ||b||_2 using the
   recursively updated residual. */
int or_pcg(int64_t n, const int32_t *rowptr, const int32_t *cols, const double *vals,
           const double *b, double *x, double rtol, int maxit, double *relres) {
    double *r = (double *)malloc((size_t)n * sizeof(double));
    double *z = (double *)malloc((size_t)n * sizeof(double));
    double *p = (double *)malloc((size_t)n * sizeof(double));
    double *q = (double *)malloc((size_t)n * sizeof(double));
    double *dinv = (double *)malloc((size_t)n * sizeof(double));
    jacobi_diag(n, rowptr, cols, vals, dinv);
    or_csr_spmv(n, rowptr, cols, vals, x, q);
    double bnorm = sqrt(dot(n, b, b));
    if (bnorm == 0.0) bnorm = 1.0;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        r[i] = b[i] - q[i];
        z[i] = dinv[i] * r[i];
        p[i] = z[i];
    }
    double rz = dot(n, r, z), rr = dot(n, r, r);
    int it = 0, status = 0;
    while (sqrt(rr) > rtol * bnorm && it < maxit) {
        or_csr_spmv(n, rowptr, cols, vals, p, q);
        double pq = dot(n, p, q);
        if (!(pq > 0.0)) {
            status = -1;
            break;
        }
        double alpha = rz / pq;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
        }
        double rz_new = dot(n, r, z);
        rr = dot(n, r, r);
        double beta = rz_new / rz;
        rz = rz_new;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        it++;
    }
    if (relres) *relres = sqrt(rr) / bnorm;
    free(r);
    free(z);
    free(p);
    free(q);
    free(dinv);
    return status ? -1 - it : it;
}

/* Jacobi right-preconditioned BiCGStab for the non-symmetric consistent
   conduction Jacobian and its transpose (adjoint). */
int or_bicgstab(int64_t n, const int32_t *rowptr, const int32_t *cols,
                const double *vals, const double *b, double *x, double rtol, int maxit,
                double *relres) {
    size_t sz = (size_t)n * sizeof(double);
    double *r = (double *)malloc(sz), *rh = (double *)malloc(sz), *p = (double *)malloc(sz);
    double *v = (double *)malloc(sz), *y = (double *)malloc(sz), *s = (double *)malloc(sz);
    double *zz = (double *)malloc(sz), *t = (double *)malloc(sz), *dinv = (double *)malloc(sz);
    jacobi_diag(n, rowptr, cols, vals, dinv);
    or_csr_spmv(n, rowptr, cols, vals, x, t);
    double bnorm = sqrt(dot(n, b, b));
    if (bnorm == 0.0) bnorm = 1.0;
    for (int64_t i = 0; i < n; i++) {
        r[i] = b[i] - t[i];
        rh[i] = r[i];
        p[i] = 0;
        v[i] = 0;
    }
    double rho = 1, alpha = 1, omega = 1, rr = dot(n, r, r);
    int it = 0, status = 0;
    while (sqrt(rr) > rtol * bnorm && it < maxit) {
        double rho_new = dot(n, rh, r);
        if (rho_new == 0.0) { status = -1; break; }
        double beta = (rho_new / rho) * (alpha / omega);
        rho = rho_new;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            p[i] = r[i] + beta * (p[i] - omega * v[i]);
            y[i] = dinv[i] * p[i];
        }
        or_csr_spmv(n, rowptr, cols, vals, y, v);
        double rv = dot(n, rh, v);
        if (rv == 0.0) { status = -1; break; }
        alpha = rho / rv;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            s[i] = r[i] - alpha * v[i];
            zz[i] = dinv[i] * s[i];
        }
        double ss = dot(n, s, s);
        if (sqrt(ss) <= rtol * bnorm) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) { x[i] += alpha * y[i]; r[i] = s[i]; }
            rr = ss;
            it++;
            break;
        }
        or_csr_spmv(n, rowptr, cols, vals, zz, t);
        double tt = dot(n, t, t), ts = dot(n, t, s);
        if (tt == 0.0) { status = -1; break; }
        omega = ts / tt;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            x[i] += alpha * y[i] + omega * zz[i];
            r[i] = s[i] - omega * t[i];
        }
        rr = dot(n, r, r);
        it++;
        if (omega == 0.0) { status = -1; break; }
    }
    if (relres) *relres = sqrt(rr) / bnorm;
    free(r); free(rh); free(p); free(v); free(y); free(s); free(zz); free(t); free(dinv);
    return status ? -1 - it : it;
}

/* ------------------------------------------------------------------------ */
/* SIMP cantilever pipeline                                                 */
/* ------------------------------------------------------------------------ */
/* ElasticityFunction (examples/structural/example_6/example_6.cpp:100-137):
   E = E0 (rho_min + (1 - rho_min) rho^p), rho_min = Emin / E0;
   dE/drho = E0 (1 - rho_min) p rho^(p-1). */
void or_simp_modulus(const or_simp_desc *d, int64_t n_el, const double *rho, double *E,
                     double *dE) {
    double rmin = d->Emin / d->E0;
    for (int64_t e = 0; e < n_el; e++) {
        if (E) E[e] = d->E0 * (rmin + (1. - rmin) * pow(rho[e], d->penal));
        if (dE) dE[e] = d->E0 * (1. - rmin) * d->penal * pow(rho[e], d->penal - 1.);
    }
}

/* Nodal density (example_6.cpp:104-137: a FIRST-order LAGRANGE "rho" field read
   through MeshFieldFunction): rho(x_q) = sum_a phi_a(x_q) rho_a at each Gauss
   point of each element, E_q = E0 (rmin + (1 - rmin) rho_q^p) and dE_q/drho_q. */
void or_simp_nodal_modulus(const or_simp_desc *d, int64_t n_el, const int32_t *conn,
                           const double *rho_nodes, double *Eq, double *dEq) {
    double rmin = d->Emin / d->E0;
    for (int64_t e = 0; e < n_el; e++)
        for (int qp = 0; qp < 8; qp++) {
            double xi[3] = {GP[qp & 1], GP[(qp >> 1) & 1], GP[(qp >> 2) & 1]}, phi[8], dref[24];
            or_hex8_shape(xi, phi, dref);
            double r = 0;
            for (int a = 0; a < 8; a++) r += phi[a] * rho_nodes[conn[e * 8 + a]];
            if (Eq) Eq[e * 8 + qp] = d->E0 * (rmin + (1. - rmin) * pow(r, d->penal));
            if (dEq) dEq[e * 8 + qp] = d->E0 * (1. - rmin) * d->penal * pow(r, d->penal - 1.);
        }
}

/* Nodal -z load on the x = max, z = 0 edge spread evenly over the node span;
   enters the residual as -F (nonlinear_implicit_assembly.cpp:189-247). */
void or_simp_load_vector(const or_simp_desc *d, double *F) {
    int64_t NX = d->nx + 1, NY = d->ny + 1, NZ = d->nz + 1;
    memset(F, 0, (size_t)(NX * NY * NZ * 3) * sizeof(double));
    int cnt = d->load_y1 - d->load_y0 + 1;
    for (int j = d->load_y0; j <= d->load_y1; j++) {
        int64_t node = d->nx + NX * j;
        F[node * 3 + 2] += -d->load_total / cnt;
    }
}

void or_simp_fixed_mask(const or_simp_desc *d, uint8_t *fixed) {
    int64_t NX = d->nx + 1, NY = d->ny + 1, NZ = d->nz + 1;
    memset(fixed, 0, (size_t)(NX * NY * NZ * 3));
    for (int64_t k = 0; k < NZ; k++)
        for (int64_t j = 0; j < NY; j++) {
            int64_t node = NX * (j + NY * k);
            fixed[node * 3] = fixed[node * 3 + 1] = fixed[node * 3 + 2] = 1;
        }
}

/* The ex-6 solve/compliance/sensitivity sequence
   (example_6.cpp:450-655, 877-939) for a structured cantilever:
   assemble K, solve K u = F, C = F.u (point loads are not in ComplianceOutput,
   compliance_output.cpp:71-102), dC/drho_e = -u_e^T dK_e/drho_e u_e (the
   compliance adjoint is -u, assembly_base.cpp:594-639). */
static int simp_solve_impl(const or_simp_desc *d, const double *rho, int nodal, double *u,
                           double *dc, or_simp_report *rep) {
    int64_t n_el = (int64_t)d->nx * d->ny * d->nz;
    int64_t n_nodes = (int64_t)(d->nx + 1) * (d->ny + 1) * (d->nz + 1);
    int64_t n = n_nodes * 3;
    double *coords = (double *)malloc((size_t)n_nodes * 3 * sizeof(double));
    int32_t *conn = (int32_t *)malloc((size_t)n_el * 8 * sizeof(int32_t));
    or_grid_hex8(d->nx, d->ny, d->nz, d->nx, d->ny, d->nz, coords, conn);
    double t0 = or_wtime();
    int32_t *rowptr = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    int64_t nnz = or_csr_pattern(8, 3, n_nodes, n_el, conn, rowptr, NULL);
    int32_t *cols = (int32_t *)malloc((size_t)nnz * sizeof(int32_t));
    or_csr_pattern(8, 3, n_nodes, n_el, conn, rowptr, cols);
    double *vals = (double *)malloc((size_t)nnz * sizeof(double));
    int32_t *color = (int32_t *)malloc((size_t)n_el * sizeof(int32_t));
    int ncol = or_color_elements(8, n_nodes, n_el, conn, color);
    const int64_t nE = nodal ? n_el * 8 : n_el;
    double *E = (double *)malloc((size_t)nE * sizeof(double));
    double *dE = (double *)malloc((size_t)nE * sizeof(double));
    if (nodal)
        or_simp_nodal_modulus(d, n_el, conn, rho, E, dE);
    else
        or_simp_modulus(d, n_el, rho, E, dE);
    uint8_t *fixed = (uint8_t *)malloc((size_t)n);
    or_simp_fixed_mask(d, fixed);
    double *F = (double *)malloc((size_t)n * sizeof(double));
    or_simp_load_vector(d, F);
    int st = assemble_hex8_impl(n_nodes, n_el, coords, conn, nodal ? NULL : E, nodal ? E : NULL,
                                d->nu, rowptr, cols, vals, fixed, ncol, color);
    double t1 = or_wtime();
    memset(u, 0, (size_t)n * sizeof(double));
    double relres = 0;
    int it = or_pcg(n, rowptr, cols, vals, F, u, d->rtol, d->maxit, &relres);
    double t2 = or_wtime();
    /* true FP64 residual */
    double *Ku = (double *)malloc((size_t)n * sizeof(double));
    or_csr_spmv(n, rowptr, cols, vals, u, Ku);
    double rn = 0, fn = 0, comp = 0;
    for (int64_t i = 0; i < n; i++) {
        rn += (F[i] - Ku[i]) * (F[i] - Ku[i]);
        fn += F[i] * F[i];
        comp += F[i] * u[i];
    }
    if (dc && nodal) {
        /* dC/drho_n = -sum over the elements of n and their Gauss points q of
           dE_q phi_n(x_q) u_e^T K1_q u_e, K1_q the unit-modulus stiffness of point q
           alone: per element first, then summed into the nodes in element order */
        double *contrib = (double *)malloc((size_t)n_el * 8 * sizeof(double));
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < n_el; e++) {
            double X[24], ue[24], df[24], eq[8], s[8];
            const int32_t *en = conn + e * 8;
            for (int a = 0; a < 8; a++)
                for (int c = 0; c < 3; c++) {
                    X[a * 3 + c] = coords[(int64_t)en[a] * 3 + c];
                    int64_t g = (int64_t)en[a] * 3 + c;
                    ue[c * 8 + a] = fixed[g] ? 0.0 : u[g];
                }
            for (int q = 0; q < 8; q++) {
                for (int k = 0; k < 8; k++) eq[k] = k == q ? 1.0 : 0.0;
                or_hex8_internal_qp(X, eq, d->nu, ue, df, NULL);
                s[q] = 0;
                for (int i = 0; i < 24; i++) s[q] += ue[i] * df[i];
            }
            for (int a = 0; a < 8; a++) {
                double acc = 0;
                for (int q = 0; q < 8; q++) {
                    double xi[3] = {GP[q & 1], GP[(q >> 1) & 1], GP[(q >> 2) & 1]}, phi[8], dref[24];
                    or_hex8_shape(xi, phi, dref);
                    acc += dE[e * 8 + q] * phi[a] * s[q];
                }
                contrib[e * 8 + a] = acc;
            }
        }
        memset(dc, 0, (size_t)n_nodes * sizeof(double));
        for (int64_t e = 0; e < n_el; e++)
            for (int a = 0; a < 8; a++) dc[conn[e * 8 + a]] -= contrib[e * 8 + a];
        free(contrib);
    } else if (dc) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < n_el; e++) {
            double X[24], ue[24], df[24];
            const int32_t *en = conn + e * 8;
            for (int a = 0; a < 8; a++)
                for (int c = 0; c < 3; c++) {
                    X[a * 3 + c] = coords[(int64_t)en[a] * 3 + c];
                    int64_t g = (int64_t)en[a] * 3 + c;
                    ue[c * 8 + a] = fixed[g] ? 0.0 : u[g];
                }
            or_hex8_internal_sens(X, dE[e], d->nu, ue, df);
            double s = 0;
            for (int i = 0; i < 24; i++) s += ue[i] * df[i];
            dc[e] = -s;
        }
    }
    double t3 = or_wtime();
    if (rep) {
        rep->iterations = it;
        rep->relres = sqrt(rn / fn);
        rep->compliance = comp;
        rep->t_assemble = t1 - t0;
        rep->t_solve = t2 - t1;
        rep->t_sens = t3 - t2;
    }
    free(coords); free(conn); free(rowptr); free(cols); free(vals); free(color);
    free(E); free(dE); free(fixed); free(F); free(Ku);
    return st ? st : (it < 0 ? it : 0);
}

int or_simp_solve(const or_simp_desc *d, const double *rho, double *u, double *dc,
                  or_simp_report *rep) {
    return simp_solve_impl(d, rho, 0, u, dc, rep);
}

/* the same with a nodal density field (n_nodes values; dc per node) */
int or_simp_solve_nodal(const or_simp_desc *d, const double *rho_nodes, double *u, double *dc,
                        or_simp_report *rep) {
    return simp_solve_impl(d, rho_nodes, 1, u, dc, rep);
}

/* ------------------------------------------------------------------------ */
/* nonlinear conduction pipeline                                            */
/* ------------------------------------------------------------------------ */
/* NonlinearSystem::solve under SNES Newton (src/base/nonlinear_system.cpp:
   209-235) with the residual/Jacobian of or_assemble_quad4_heat; then the
   mean-temperature output, its adjoint (NonlinearSystem::adjoint_solve,
   :798-847: J^T lambda = -dq/dT) and the sensitivities
   dq/dp = lambda . dR/dp (AssemblyBase::calculate_output_adjoint_sensitivity,
   src/base/assembly_base.cpp:555-590). */
int or_heat_solve(const or_heat_desc *d, const double *s_elem, const double *q_elem,
                  double *T, double *dq_ds, or_heat_report *rep) {
    double t0 = or_wtime();
    int nx = d->nx, ny = d->ny;
    int64_t n_el = (int64_t)nx * ny, n = (int64_t)(nx + 1) * (ny + 1);
    double *coords = (double *)malloc((size_t)n * 2 * sizeof(double));
    int32_t *conn = (int32_t *)malloc((size_t)n_el * 4 * sizeof(int32_t));
    or_grid_quad4(nx, ny, d->lx, d->ly, coords, conn);
    int32_t *rowptr = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    int64_t nnz = or_csr_pattern(4, 1, n, n_el, conn, rowptr, NULL);
    int32_t *cols = (int32_t *)malloc((size_t)nnz * sizeof(int32_t));
    or_csr_pattern(4, 1, n, n_el, conn, rowptr, cols);
    double *vals = (double *)malloc((size_t)nnz * sizeof(double));
    uint8_t *fixed = (uint8_t *)calloc((size_t)n, 1);
    for (int j = 0; j <= ny; j++) fixed[(int64_t)(nx + 1) * j] = 1;
    int32_t *ce = (int32_t *)malloc((size_t)(ny > 0 ? ny : 1) * sizeof(int32_t));
    int32_t *cs = (int32_t *)malloc((size_t)(ny > 0 ? ny : 1) * sizeof(int32_t));
    for (int j = 0; j < ny; j++) {
        ce[j] = (nx - 1) + nx * j;
        cs[j] = 1;
    }
    double *R = (double *)malloc((size_t)n * sizeof(double));
    double *dT = (double *)malloc((size_t)n * sizeof(double));
    memset(T, 0, (size_t)n * sizeof(double));
    int newton = 0, kry = 0, st = 0;
    double r0 = -1, rn = 0;
    for (newton = 0; newton <= d->max_newton; newton++) {
        or_assemble_quad4_heat(n, n_el, coords, conn, d->k0, d->beta, s_elem, d->h, q_elem,
                               ny, ce, cs, d->hc, d->Tinf, T, d->consistent, rowptr, cols,
                               vals, R, fixed);
        rn = sqrt(dot(n, R, R));
        if (r0 < 0) r0 = rn;
        if (rn <= d->newton_rtol * r0 || newton == d->max_newton) break;
        for (int64_t i = 0; i < n; i++) { R[i] = -R[i]; dT[i] = 0; }
        double rr;
        int it = d->krylov ? or_bicgstab(n, rowptr, cols, vals, R, dT, d->rtol, d->maxit, &rr)
                           : or_pcg(n, rowptr, cols, vals, R, dT, d->rtol, d->maxit, &rr);
        if (it < 0) { st = -2; break; }
        kry += it;
        for (int64_t i = 0; i < n; i++) T[i] += dT[i];
    }
    /* output q = (1/area) int T; dq/dT_i = (1/area) int phi_i */
    double area = d->lx * d->ly, qv = 0;
    double *dqdT = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t e = 0; e < n_el; e++) {
        double X[8], phi[4], dphi[8], JxW;
        const int32_t *en = conn + e * 4;
        for (int a = 0; a < 4; a++) {
            X[a * 2] = coords[(int64_t)en[a] * 2];
            X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
        }
        for (int qp = 0; qp < 4; qp++) {
            quad4_qp(X, qp, phi, dphi, &JxW);
            for (int a = 0; a < 4; a++) {
                qv += JxW * phi[a] * T[en[a]] / area;
                dqdT[en[a]] += JxW * phi[a] / area;
            }
        }
    }
    /* adjoint: J^T lambda = -dq/dT on free dofs (consistent Jacobian at T) */
    or_assemble_quad4_heat(n, n_el, coords, conn, d->k0, d->beta, s_elem, d->h, q_elem, ny,
                           ce, cs, d->hc, d->Tinf, T, 1, rowptr, cols, vals, NULL, fixed);
    int32_t *rpt = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *ct = (int32_t *)malloc((size_t)nnz * sizeof(int32_t));
    double *vt = (double *)malloc((size_t)nnz * sizeof(double));
    or_csr_transpose(n, rowptr, cols, vals, rpt, ct, vt);
    double *lam = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < n; i++) R[i] = fixed[i] ? 0.0 : -dqdT[i];
    double rr;
    int it = or_bicgstab(n, rpt, ct, vt, R, lam, d->rtol, d->maxit, &rr);
    if (it < 0) st = -3;
    /* sensitivities: k0 (global) and per-element scale s_e */
    double dk0 = 0;
    for (int64_t e = 0; e < n_el; e++) {
        double X[8], Te[4], df[4];
        const int32_t *en = conn + e * 4;
        double se = s_elem ? s_elem[e] : 1.0;
        for (int a = 0; a < 4; a++) {
            X[a * 2] = coords[(int64_t)en[a] * 2];
            X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
            Te[a] = T[en[a]];
        }
        or_quad4_heat_internal_sens(X, se, se * d->beta, d->h, Te, df);
        double s = 0;
        for (int a = 0; a < 4; a++) s += lam[en[a]] * df[a];
        dk0 += s;
        if (dq_ds) {
            or_quad4_heat_internal_sens(X, d->k0, d->k0 * d->beta, d->h, Te, df);
            s = 0;
            for (int a = 0; a < 4; a++) s += lam[en[a]] * df[a];
            dq_ds[e] = s;
        }
    }
    if (rep) {
        rep->newton_iterations = newton;
        rep->krylov_iterations = kry;
        rep->residual_norm = rn;
        rep->mean_temperature = qv;
        rep->dq_dk0 = dk0;
        rep->t_total = or_wtime() - t0;
    }
    free(coords); free(conn); free(rowptr); free(cols); free(vals); free(fixed);
    free(ce); free(cs); free(R); free(dT); free(dqdT); free(rpt); free(ct); free(vt); free(lam);
    return st;
}

/* ------------------------------------------------------------------ density filter
   MAST::FilterBase (src/level_set/filter_base.cpp): the weights of point i are
   w_ij = (r - d_ij) / sum_k (r - d_ik) over every point j with d_ij <= r
   (`_init`, the linear search, :378-437, normalised at :429-435); the
   filtered value of a design-variable point is sum_j w_ij x_j, any other point
   keeps its input value (compute_filtered_values, :58-95).  Plain O(n^2)
   search over the points, as the reference's linear search does. */
int or_filter_points(int64_t n, int dim, const double *xyz, double r, const uint8_t *dv,
                     const double *in, double *out, int transpose) {
    if (n <= 0 || r <= 0.0) return -1;
    double *S = (double *)calloc((size_t)n, sizeof(double));
    if (!S) return -2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double s = 0.0;
        for (int64_t j = 0; j < n; j++) {
            double d2 = 0.0;
            for (int c = 0; c < dim; c++) {
                const double t = xyz[i * dim + c] - xyz[j * dim + c];
                d2 += t * t;
            }
            if (d2 <= r * r) s += r - sqrt(d2);
        }
        S[i] = s;
    }
    if (!transpose) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            if (dv && !dv[i]) { out[i] = in[i]; continue; }
            double acc = 0.0;
            for (int64_t j = 0; j < n; j++) {
                double d2 = 0.0;
                for (int c = 0; c < dim; c++) {
                    const double t = xyz[i * dim + c] - xyz[j * dim + c];
                    d2 += t * t;
                }
                if (d2 <= r * r) acc += (r - sqrt(d2)) / S[i] * in[j];
            }
            out[i] = acc;
        }
    } else {
        /* out_j = sum_i [dv_i] w_ij in_i + [!dv_j] in_j */
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n; j++) {
            double acc = (dv && !dv[j]) ? in[j] : 0.0;
            for (int64_t i = 0; i < n; i++) {
                if (dv && !dv[i]) continue;
                double d2 = 0.0;
                for (int c = 0; c < dim; c++) {
                    const double t = xyz[i * dim + c] - xyz[j * dim + c];
                    d2 += t * t;
                }
                if (d2 <= r * r) acc += (r - sqrt(d2)) / S[i] * in[i];
            }
            out[j] = acc;
        }
    }
    free(S);
    return 0;
}

/* element centroids of a structured grid (spacing hx, hy, hz; nz = 0: 2D) */
void or_grid_centroids(int nx, int ny, int nz, double hx, double hy, double hz, double *xyz) {
    const int dim = nz > 0 ? 3 : 2, NZ = nz > 0 ? nz : 1;
    int64_t e = 0;
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++, e++) {
                xyz[e * dim] = (i + 0.5) * hx;
                xyz[e * dim + 1] = (j + 0.5) * hy;
                if (dim == 3) xyz[e * dim + 2] = (k + 0.5) * hz;
            }
}
