/*
 * mast_oracle.h -- FP64 CPU restatement of MAST's HEX8/QUAD4 element,
 * assembly, Krylov and sensitivity arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests compare the CUDA product (libmastgpu.so)
 * against this library, and it is the timed CPU baseline; nothing in the product links,
 * loads or calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm use it.
 *
 * Parity status: the material matrices are pinned to the hand-computed truth
 * values of the reference's own unit tests (tests/material/
 * mast_isotropic_material.cpp:272-445, 611-708); the QUAD4 membrane element is
 * pinned by the property checks of tests/element/structural/2D/quad4/ files
 * (6th-order finite-difference Jacobian, symmetry, rigid modes, fixed
 * displacement vector).  The reference ships no golden vectors for HEX8,
 * the heat element, assembly, solves or sensitivities; those are pinned by
 * finite differences, rigid-body modes, patch tests, an analytic 1D
 * conduction solution and scipy direct solves (see tests/test_oracle_*.py).
 *
 * Conventions shared with the reference:
 *  - element DOF order is variable-blocked [u0..u7, v0..v7, w0..w7]
 *    (src/numerics/fem_operator_matrix.h:262-300);
 *  - Voigt order [xx, yy, zz, xy, yz, zx] with engineering shear
 *    (src/elasticity/solid_element_3d.cpp:1272-1304);
 *  - libMesh LAGRANGE FIRST node ordering and 2-point Gauss per direction
 *    (src/mesh/fe_base.cpp:103-107, libMesh ext.);
 *  - residual R = f_int - f_ext; point loads enter as -F
 *    (src/base/nonlinear_implicit_assembly.cpp:189-247).
 * Global numbering is node-interleaved: dof = dpn*node + component.
 */
#ifndef MAST_ORACLE_H
#define MAST_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* material / reference element */
void or_iso_stiffness_3d(double E, double nu, double C[36]);
void or_iso_stiffness_2d(double E, double nu, int plane_stress, double C[9]);
void or_hex8_shape(const double xi[3], double phi[8], double dphi[24]);
void or_quad4_shape(const double xi[2], double phi[4], double dphi[8]);

/* element routines (var-blocked order; K may be NULL) */
int or_hex8_internal(const double X[24], double E, double nu, const double u[24],
                     double f[24], double K[576]);
int or_hex8_internal_qp(const double X[24], const double Eq[8], double nu, const double u[24],
                        double f[24], double K[576]);
/* HEX8 total-Lagrangian Green-Lagrange element (nonlinear-strain branch):
   f = int B_L^T S, K = int (B_L^T C B_L + geometric stiffness); var-blocked dofs */
int or_hex8_internal_gl(const double X[24], double E, double nu, const double u[24],
                        double f[24], double K[576]);
/* Gauss-point stress (Voigt), von Mises, JxW and d sigma / d u (nullable, 8 x 6 x 24) */
/* side loads: HEX8 pressure as an external load (var-blocked), QUAD4 heat flux residual */
void or_hex8_pressure(const double X[24], int side, double p, double f[24]);
void or_quad4_heat_flux(const double X[8], int side, double flux, double th, double f[4]);
int or_hex8_stress(const double X[24], double E, double nu, const double u[24], int nonlinear,
                   double sig[48], double vm[8], double JxW_out[8], double *dsig);
int or_hex8_internal_sens(const double X[24], double dE, double nu,
                          const double u[24], double df[24]);
int or_quad4_membrane_internal(const double X[8], double E, double nu, double h,
                               const double u[8], double f[8], double K[64]);
int or_quad4_heat_internal(const double X[8], double k0, double beta, double s,
                           double h, const double T[4], int consistent,
                           double f[4], double K[16]);
int or_quad4_heat_internal_sens(const double X[8], double a, double b, double h,
                                const double T[4], double df[4]);
void or_quad4_heat_convection(const double X[8], int side, double hc, double Tinf,
                              double th, const double T[4], double f[4], double K[16]);
void or_quad4_heat_source(const double X[8], double q, double th, double f[4]);

/* structured meshes (libMesh build_cube / build_square numbering) */
void or_grid_hex8(int nx, int ny, int nz, double lx, double ly, double lz,
                  double *coords, int32_t *conn);
void or_grid_quad4(int nx, int ny, double lx, double ly, double *coords, int32_t *conn);

/* sparse pattern, colouring, SpMV */
int64_t or_csr_pattern(int npe, int dpn, int64_t n_nodes, int64_t n_elems,
                       const int32_t *conn, int32_t *rowptr, int32_t *cols);
int or_color_elements(int npe, int64_t n_nodes, int64_t n_elems, const int32_t *conn,
                      int32_t *color);
void or_csr_spmv(int64_t n, const int32_t *rowptr, const int32_t *cols,
                 const double *vals, const double *x, double *y);
void or_csr_transpose(int64_t n, const int32_t *rowptr, const int32_t *cols,
                      const double *vals, int32_t *rowptr_t, int32_t *cols_t,
                      double *vals_t);

/* assembly into a CSR with a given pattern; fixed[dof]!=0 -> identity row/col */
int or_assemble_hex8(int64_t n_nodes, int64_t n_elems, const double *coords,
                     const int32_t *conn, const double *E_elem, double nu,
                     const int32_t *rowptr, const int32_t *cols, double *vals,
                     const uint8_t *fixed, int n_colors, const int32_t *color);
int or_assemble_hex8_qp(int64_t n_nodes, int64_t n_elems, const double *coords,
                     const int32_t *conn, const double *E_qp, double nu,
                     const int32_t *rowptr, const int32_t *cols, double *vals,
                     const uint8_t *fixed, int n_colors, const int32_t *color);
int or_assemble_quad4_membrane(int64_t n_nodes, int64_t n_elems, const double *coords,
                               const int32_t *conn, const double *E_elem, double nu,
                               double h, const int32_t *rowptr, const int32_t *cols,
                               double *vals, const uint8_t *fixed);
int or_assemble_quad4_heat(int64_t n_nodes, int64_t n_elems, const double *coords,
                           const int32_t *conn, double k0, double beta,
                           const double *s_elem, double h, const double *q_elem,
                           int64_t n_conv, const int32_t *conv_elem,
                           const int32_t *conv_side, double hc, double Tinf,
                           const double *T, int consistent,
                           const int32_t *rowptr, const int32_t *cols, double *vals,
                           double *R, const uint8_t *fixed);
/* Green-Lagrange HEX8: R = f_int(u) - F (F nullable), tangent into vals (nullable) */
int or_assemble_hex8_gl(int64_t n_nodes, int64_t n_elems, const double *coords,
                        const int32_t *conn, const double *E_elem, double nu, const double *u,
                        const double *F, const int32_t *rowptr, const int32_t *cols,
                        double *vals, double *R, const uint8_t *fixed);

/* Krylov (Jacobi preconditioned); return iterations, <0 on breakdown */
int or_pcg(int64_t n, const int32_t *rowptr, const int32_t *cols, const double *vals,
           const double *b, double *x, double rtol, int maxit, double *relres);
int or_bicgstab(int64_t n, const int32_t *rowptr, const int32_t *cols,
                const double *vals, const double *b, double *x, double rtol, int maxit,
                double *relres);

/* SIMP cantilever pipeline (structured HEX8 grid, x=0 clamp, -z load on the
   x=max, z=0 edge over node span [y0,y1]) */
typedef struct {
    int nx, ny, nz;
    double E0, Emin, nu, penal;
    int load_y0, load_y1;  /* inclusive node range of the loaded edge */
    double load_total;     /* total -z load (1.0) */
    double rtol;
    int maxit;
} or_simp_desc;

typedef struct {
    int iterations;
    double relres;          /* ||f - K u|| / ||f|| in FP64 */
    double compliance;      /* f . u */
    double t_assemble, t_solve, t_sens;  /* seconds */
} or_simp_report;

int or_simp_solve(const or_simp_desc *d, const double *rho, double *u, double *dc,
                  or_simp_report *rep);
/* nodal density field (MeshFieldFunction, trilinear per element): rho_nodes has
   (nx+1)(ny+1)(nz+1) values, dc one per node */
int or_simp_solve_nodal(const or_simp_desc *d, const double *rho_nodes, double *u, double *dc,
                        or_simp_report *rep);
void or_simp_nodal_modulus(const or_simp_desc *d, int64_t n_el, const int32_t *conn,
                           const double *rho_nodes, double *Eq, double *dEq);
void or_simp_load_vector(const or_simp_desc *d, double *F);
void or_simp_fixed_mask(const or_simp_desc *d, uint8_t *fixed);
void or_simp_modulus(const or_simp_desc *d, int64_t n_el, const double *rho, double *E,
                     double *dE);

/* nonlinear conduction pipeline (QUAD4 square, T=0 at x=0, convection at x=1,
   source q_elem, k = k0 (1 + beta T) s_e h) */
typedef struct {
    int nx, ny;
    double lx, ly;
    double k0, beta, h;
    double hc, Tinf;
    double rtol;           /* inner Krylov tolerance */
    double newton_rtol;    /* ||R|| / ||R0|| stop */
    int maxit, max_newton;
    int consistent;        /* 1: dk/dT Jacobian term; 0: reference Jacobian */
    int krylov;            /* 0: PCG, 1: BiCGStab */
} or_heat_desc;

typedef struct {
    int newton_iterations;
    int krylov_iterations;
    double residual_norm;
    double mean_temperature;
    double dq_dk0;
    double t_total;
} or_heat_report;

int or_heat_solve(const or_heat_desc *d, const double *s_elem, const double *q_elem,
                  double *T, double *dq_ds, or_heat_report *rep);

/* density filter of MAST::FilterBase over points (transpose = 1: the chain
   rule F^T); element centroids of a structured grid */
int or_filter_points(int64_t n, int dim, const double *xyz, double r, const uint8_t *dv,
                     const double *in, double *out, int transpose);
void or_grid_centroids(int nx, int ny, int nz, double hx, double hy, double hz, double *xyz);

/* bounded-sample timers used by the CPU baseline */
double or_wtime(void);
int or_max_threads(void);
void or_set_threads(int n);
void or_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
