/*
 * mastgpu.h -- C ABI of the GB300-native MAST finite-element hot path.
 *
 * One opaque handle (mg_problem) owns one mesh, its design/material state, the
 * device CSR system and the Krylov workspace on one GPU and one CUDA stream.
 * All buffers passed in are caller-owned HOST buffers unless a name ends in
 * _device.  Every entry point returns an mg_status (0 = MG_OK); no exception
 * crosses the ABI.  One handle must be used from one thread at a time;
 * distinct handles are independent.
 *
 * Reference interfaces each entry point replaces (paths in the MAST tree):
 *   mg_problem_create          libMesh EquationSystems/DofMap set-up done by
 *                              MAST::StructuralSystemInitialization
 *                              (src/elasticity/structural_system_initialization.cpp:29-42),
 *                              MAST::PhysicsDisciplineBase Dirichlet/loads
 *                              (src/base/physics_discipline_base.cpp:218-229)
 *                              and the property cards
 *                              (src/property_cards/isotropic_element_property_card_3D.cpp:422-443)
 *   mg_set_design              the SIMP density field behind
 *                              ElasticityFunction (examples/structural/example_6/example_6.cpp:100-137)
 *   mg_residual_and_jacobian   MAST::NonlinearImplicitAssembly::residual_and_jacobian
 *                              (src/base/nonlinear_implicit_assembly.cpp:64-266,
 *                              declared src/base/nonlinear_implicit_assembly.h:99-104)
 *   mg_element_matrices        MAST::NonlinearImplicitAssemblyElemOperations::elem_calculations
 *                              (src/base/nonlinear_implicit_assembly_elem_operations.h:50-105;
 *                              src/elasticity/structural_nonlinear_assembly.cpp:112-139)
 *   mg_solve                   MAST::NonlinearSystem::solve
 *                              (src/base/nonlinear_system.cpp:209-235) with the
 *                              libMesh/PETSc SNES + KSP it drives
 *   mg_sensitivity_assemble    MAST::NonlinearImplicitAssembly::sensitivity_assemble
 *                              (src/base/nonlinear_implicit_assembly.cpp:515-686)
 *   mg_compliance              MAST::ComplianceOutput + AssemblyBase::calculate_output /
 *                              calculate_output_adjoint_sensitivity_multiple_parameters_no_direct
 *                              (src/elasticity/compliance_output.cpp:71-296,
 *                              src/base/assembly_base.cpp:253-333, 594-639)
 *   mg_mean_temperature        an OutputAssemblyElemOperations subclass
 *                              (src/base/output_assembly_elem_operations.h:64-250)
 *                              with NonlinearSystem::adjoint_solve
 *                              (src/base/nonlinear_system.cpp:798-847) and
 *                              AssemblyBase::calculate_output_adjoint_sensitivity
 *                              (src/base/assembly_base.cpp:555-590)
 */
#ifndef MASTGPU_H
#define MASTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_ABI_VERSION 1

typedef enum mg_status {
    MG_OK = 0,
    MG_EINVAL = -1,      /* bad argument, malformed mesh/offset table, NaN input */
    MG_ENOMEM = -2,      /* device allocation failed */
    MG_ENOCONV = -3,     /* iteration cap reached before the tolerance */
    MG_EBREAKDOWN = -4,  /* Krylov breakdown (p^T A p <= 0, rho = 0, ...) */
    MG_ENAN = -5,        /* NaN/Inf met in a device reduction */
    MG_ETIMEDOUT = -6,   /* host wait exceeded its wall-clock limit */
    MG_ECUDA = -7,       /* CUDA runtime error (mg_last_error() has the text) */
    MG_ENOTSUP = -8,     /* operation not available for this physics/mesh */
    MG_EBUSY = -9,       /* admission refused / queue full */
    MG_EBADELEM = -10    /* non-positive Jacobian determinant in an element */
} mg_status;

typedef enum mg_physics {
    MG_PHYSICS_ELASTICITY_HEX8 = 0, /* StructuralElement3D, 3 translational dofs/node */
    MG_PHYSICS_MEMBRANE_QUAD4 = 1,  /* StructuralElement2D membrane, 2 dofs/node */
    MG_PHYSICS_HEAT_QUAD4 = 2       /* HeatConductionElementBase, 1 dof/node */
} mg_physics;

typedef enum mg_precision {
    MG_PLAIN_FP64 = 0,  /* FP64 element quadrature, CSR, Krylov */
    MG_MIXED_TF32 = 1,  /* matrix-free tcgen05 TF32 operator, FP32 CG, FP64 refinement */
    MG_MIXED_BF16 = 2,  /* as above with BF16 operands (FP32 accumulation) */
    MG_MIXED_TF32X3 = 3, /* split TF32: (u_hi + u_lo)(K_hi + K_lo) minus the lo*lo term,
                            three TF32 products per element, FP32 accumulation */
    MG_MIXED_BF16X3 = 4  /* split BF16, three BF16 products, FP32 accumulation */
} mg_precision;

typedef enum mg_krylov { MG_KRYLOV_CG = 0, MG_KRYLOV_BICGSTAB = 1 } mg_krylov;

typedef struct mg_problem mg_problem;

typedef struct mg_mesh_desc {
    int32_t physics;        /* mg_physics */
    int32_t reserved0;
    int64_t n_nodes;
    int64_t n_elems;
    const double *coords;   /* n_nodes x dim (3 for HEX8, 2 for QUAD4), node-major */
    const int32_t *conn;    /* n_elems x npe, libMesh local node order */
    int32_t grid_nx, grid_ny, grid_nz; /* structured-grid dims if the mesh is the
                                          unit-spaced libMesh build_cube grid, else 0 */
    int32_t reserved1;
} mg_mesh_desc;

typedef struct mg_material_desc {
    double E0, Emin, nu, penal; /* E(rho) = E0 (rmin + (1 - rmin) rho^p), rmin = Emin/E0 */
    double thickness;           /* 2D section thickness h */
    double k0, k_beta;          /* k(T) = k0 (1 + k_beta T) s_e */
} mg_material_desc;

typedef struct mg_bc_desc {
    int64_t n_fixed;             /* homogeneous Dirichlet dofs (dof = dpn*node + comp) */
    const int64_t *fixed_dofs;
    int64_t n_point_loads;       /* nodal loads F, enter the residual as -F */
    const int64_t *load_dofs;
    const double *load_values;
    int64_t n_conv;              /* convection sides (heat) */
    const int32_t *conv_elems;
    const int32_t *conv_sides;   /* libMesh side numbering */
    double conv_h, conv_Tinf;
    const double *source_elem;   /* per-element volume heat source q (nullable) */
} mg_bc_desc;

typedef struct mg_solve_opts {
    int32_t precision;       /* mg_precision */
    int32_t krylov;          /* mg_krylov (plain form) */
    int32_t max_iterations;  /* Krylov cap per linear solve */
    int32_t max_newton;      /* Newton cap (1 step suffices for linear physics) */
    double rtol;             /* ||b - A x|| / ||b|| target (FP64 residual) */
    double newton_rtol;      /* ||R|| / ||R0|| Newton stop */
    int32_t consistent_jacobian; /* heat: include the dk/dT term */
    int32_t max_refinements; /* mixed: FP64 refinement cap */
    double inner_rtol;       /* mixed: FP32 inner CG tolerance per refinement */
    double timeout_s;        /* host wall-clock limit for the solve (0 = none) */
    int32_t warm_start;      /* 1: start from the resident solution */
    int32_t graph_chunk;     /* Krylov iterations per captured CUDA graph (0 = default) */
    int32_t preconditioner;  /* mixed form: MG_PC_MULTIGRID (default) or MG_PC_JACOBI;
                                the plain form is Jacobi-preconditioned */
    int32_t smooth_degree;   /* multigrid: Chebyshev degree of the smoothers (0 = 2) */
    int32_t coarse_degree;   /* multigrid: Chebyshev degree on the coarsest grid (0 = 8) */
    int32_t reserved;
} mg_solve_opts;

#define MG_PC_JACOBI 0
#define MG_PC_MULTIGRID 1

typedef struct mg_solve_report {
    int32_t status;
    int32_t newton_iterations;
    int32_t krylov_iterations;
    int32_t refinements;
    double relres;           /* final FP64 ||b - A x|| / ||b|| */
    double residual_norm;    /* final nonlinear ||R|| */
    double seconds;
} mg_solve_report;

/* ---- library ---- */
int mg_version(void);
const char *mg_status_string(int status);
const char *mg_last_error(void);
int mg_device_info(char *name, int name_len, int *sm_count, int *cc_major, int *cc_minor);
void mg_default_solve_opts(mg_solve_opts *opts);

/* ---- problem set-up ---- */
int mg_problem_create(const mg_mesh_desc *mesh, const mg_material_desc *mat,
                      const mg_bc_desc *bc, mg_problem **out);
void mg_problem_destroy(mg_problem *p);
int mg_problem_info(const mg_problem *p, int64_t *n_dofs, int64_t *nnz, int32_t *n_colors);
void *mg_problem_stream(mg_problem *p); /* the handle's cudaStream_t */

/* ---- design / properties ---- */
int mg_set_design(mg_problem *p, const double *rho_elem);
int mg_set_design_device(mg_problem *p, const double *rho_elem_device);
int mg_set_elem_scale(mg_problem *p, const double *s_elem);

/* ---- assembly (plain FP64) ---- */
int mg_residual_and_jacobian(mg_problem *p, const double *X, double *R, int assemble_jacobian);
int mg_get_csr(mg_problem *p, int32_t *rowptr, int32_t *cols, double *vals);
int mg_element_matrices(mg_problem *p, const double *X, int64_t first, int64_t count,
                        double *Ke, double *fe);
int mg_spmv(mg_problem *p, const double *x, double *y);

/* ---- solve ---- */
int mg_solve(mg_problem *p, const mg_solve_opts *opts, double *X, mg_solve_report *rep);
int mg_get_solution(mg_problem *p, double *X);
const double *mg_solution_device(mg_problem *p);

/* ---- outputs and sensitivities ---- */
int mg_sensitivity_assemble(mg_problem *p, const double *X, int32_t param_kind,
                            int64_t param_index, double *dRdp);
int mg_compliance(mg_problem *p, const double *X, double *compliance, double *dc_drho);
int mg_mean_temperature(mg_problem *p, const double *T, const mg_solve_opts *opts,
                        double *qbar, double *dq_dk0, double *dq_ds);

/* ---- testing hook ---- */
/* Host-side fault injection: the countdown-th next device allocation made by
   the library reports MG_ENOMEM (-1 disables).  No GPU fault is involved. */
void mg_debug_fail_alloc_after(int countdown);
/* One application of the mixed-precision matrix-free operator y = A x
   (precision MG_MIXED_TF32 / MG_MIXED_BF16; x must be zero on Dirichlet dofs). */
int mg_debug_matfree_apply(mg_problem *p, int precision, const double *x, double *y);

/* ---- device-resident outputs and diagnostics ---- */
/* Compliance f.u (to *compliance on the host) and dC/drho_e into the handle's
   device buffer mg_sensitivities_device(p), from the resident solution. */
int mg_compliance_resident(mg_problem *p, double *compliance);
const double *mg_sensitivities_device(mg_problem *p);
/* Kernel launches issued by the library so far (graph nodes included). */
long long mg_launch_count(void);
/* Enqueues `reps` launches of the dominant Krylov kernel on the handle's stream
   without synchronising (for event timing): the fused CSR SpMV of the CG step
   (MG_PLAIN_FP64) or the tensor-core brick operator (MG_MIXED_*). */
int mg_debug_launch_apply(mg_problem *p, int precision, int reps);

/* ---- allocation-free solve ---- */
/* No counterpart in the reference (MAST hands its linear systems to PETSc).
   Jacobi-preconditioned CG on a caller-owned CSR (n rows, int32 rowptr/cols,
   FP64 values, all device pointers) with right-hand side b and initial guess /
   solution x (device pointers), to ||b - A x|| <= rtol ||b||, enqueued on
   `stream` (a cudaStream_t; NULL = default stream).  It is for callers that
   cannot call cudaMalloc: code that must not allocate after start-up (a
   request loop running inside a fixed device-memory budget) and host
   applications whose own pool owns all device memory.  The library allocates
   nothing here: its scratch is one static device array of about 6.3 MB that
   every GPU loading the library holds until exit, which limits n to
   MG_STATIC_PCG_MAX_N (larger n returns MG_EINVAL).  The first call on a
   device looks the array's address up (cudaGetSymbolAddress); make that first
   call before any stream capture.  All calls share the array, so calls that
   overlap on the GPU race; serialise them.  Returns MG_OK, MG_ENOCONV,
   MG_EBREAKDOWN or MG_ENAN; *iterations and *relres (nullable) report the
   iteration count and final relative residual. */
#define MG_STATIC_PCG_MAX_N 131072
int mg_pcg_csr_static(int64_t n, const int32_t *rowptr, const int32_t *cols, const double *vals,
                      const double *b, double *x, double rtol, int32_t max_iterations,
                      void *stream, int32_t *iterations, double *relres);

/* parameter kinds for mg_sensitivity_assemble */
#define MG_PARAM_DENSITY 0      /* rho_e of element param_index (elasticity) */
#define MG_PARAM_K0 1           /* conductivity k0 (heat) */
#define MG_PARAM_ELEM_SCALE 2   /* conductivity scale s_e of element param_index (heat) */

#ifdef __cplusplus
}
#endif
#endif /* MASTGPU_H */
