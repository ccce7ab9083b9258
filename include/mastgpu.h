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
 *   mg_ks_stress               MAST::KSStressStrainOutput (src/elasticity/ks_stress_output.cpp)
 *                              over StructuralElement3D::calculate_stress
 *                              (src/elasticity/solid_element_3d.cpp:1147-1270), with the
 *                              adjoint sensitivity of examples/structural/example_6/example_6.cpp:798-874
 *   mg_adjoint_solve           MAST::NonlinearSystem::adjoint_solve
 *                              (src/base/nonlinear_system.cpp:798-847)
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
    MG_PHYSICS_HEAT_QUAD4 = 2,      /* HeatConductionElementBase, 1 dof/node */
    MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR = 3 /* StructuralElement3D with the section's strain
                                                type MAST::NONLINEAR_STRAIN (Green-Lagrange,
                                                total Lagrangian; element_property_card_base.h:
                                                36-41): Newton on the plain FP64 form */
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
    int32_t vec_blocks_per_sm; /* mixed form: CTAs per SM of the vector kernels (0 = 8) */
    int32_t smoother_operator; /* multigrid level operator: MG_SMOOTHER_FACTORED (0, default:
                                  FP32 on the CUDA cores, factored element stiffness) or
                                  MG_SMOOTHER_TENSOR (the tensor-core operator, single pass
                                  of the CG operator's input type) */
} mg_solve_opts;

#define MG_SMOOTHER_FACTORED 0
#define MG_SMOOTHER_TENSOR 1

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

/* ---- side loads ---- */
/* Side boundary conditions (PhysicsDisciplineBase side loads), replacing earlier ones:
   HEX8 physics: "pressure" p on element face `side` (libMesh Hex8 side numbering),
   external load +int phi p n dA with n the outward reference normal
   (StructuralElement3D::surface_pressure_residual, solid_element_3d.cpp:815-876);
   heat: "heat_flux" q_n on element edge `side`, residual +int phi q_n th ds
   (surface_flux_residual, heat_conduction_elem_base.cpp:876-913).  The load is
   assembled on the GPU into the problem's load vector with the point loads.
   MG_ENOTSUP for the membrane physics. */
int mg_set_side_loads(mg_problem *p, int64_t n, const int32_t *elems, const int32_t *sides,
                      const double *values);

/* ---- design / properties ---- */
int mg_set_design(mg_problem *p, const double *rho_elem);
int mg_set_design_device(mg_problem *p, const double *rho_elem_device);
/* Nodal SIMP density field, n_nodes values in [0,1]: the design of MAST example 6,
   a FIRST-order LAGRANGE "rho" read through MeshFieldFunction
   (examples/structural/example_6/example_6.cpp:104-137, 250-252; MeshFieldFunction,
   src/base/mesh_field_function.cpp:205-350).  The modulus is evaluated at each
   Gauss point from the trilinear field there, E = E0 (rmin + (1 - rmin) rho^p);
   mg_compliance then returns dC/drho per node (n_nodes values).  Linear-strain HEX8
   on the plain FP64 path: the mixed-precision solve, the KS stress output and the
   per-element sensitivity entry points answer MG_ENOTSUP while a nodal field is
   set (mg_set_design goes back to element densities). */
int mg_set_design_nodal(mg_problem *p, const double *rho_nodes);
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
/* compliance C = F.X; dc_drho (nullable) by the adjoint: lambda = -X for the linear
   form, K_T(X) lambda = F on the GPU for MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR; one value
   per element, or per node after mg_set_design_nodal */
int mg_compliance(mg_problem *p, const double *X, double *compliance, double *dc_drho);
/* KS-aggregated von Mises stress over every element (KSStressStrainOutput,
   ks_stress_output.cpp:41-99) at X (host, nullable: the resident solution):
   ks = ln(sum_qp exp(p_ks (vm - sigma0)/sigma0) JxW / sum_qp JxW) / p_ks with the stress
   of E(rho) at the SIMP exponent stress_penalty (<= 0: the material's), max_vm the
   largest Gauss-point von Mises stress; dks_drho (nullable, n_elems) the total density
   derivative as example_6.cpp:798-874 forms it: lambda . dR/drho with
   K(X)^T lambda = -dks/dX (the tangent for the nonlinear strain), plus the direct term
   through the stress modulus.  HEX8 physics only. */
int mg_ks_stress(mg_problem *p, const double *X, double p_ks, double sigma0, double stress_penalty,
                 double *ks, double *max_vm, double *dks_drho);
/* J(X)^T lambda = rhs with the consistent Jacobian at X (host vectors; constrained
   rows give lambda = 0); the Krylov method of opts (BiCGStab for heat) */
int mg_adjoint_solve(mg_problem *p, const double *X, const double *rhs, const mg_solve_opts *opts,
                     double *lambda);
/* J(X) du_dp = -dR/dp for one parameter (kind, index as mg_sensitivity_assemble) with the
   consistent Jacobian at X: the forward sensitivity of the solution, as
   MAST::NonlinearSystem::sensitivity_solve (src/base/nonlinear_system.cpp:741-794,
   declared src/base/nonlinear_system.h:142) forms it for
   AssemblyBase::calculate_output_direct_sensitivity (src/base/assembly_base.cpp:434-520).
   Constrained rows give du_dp = 0; the Krylov method of opts (BiCGStab for heat). */
int mg_sensitivity_solve(mg_problem *p, const double *X, int32_t kind, int64_t index,
                         const mg_solve_opts *opts, double *du_dp);
/* dq/dX of an output at X (host, nullable: the resident solution), zero on constrained
   dofs: MAST::AssemblyBase::calculate_output_derivative (src/base/assembly_base.cpp:336-429).
   MG_OUTPUT_COMPLIANCE: C = F.X, dC/dX = F (structural physics); MG_OUTPUT_MEAN_TEMPERATURE:
   the lumped weights of (1/|Omega|) int T (heat). */
#define MG_OUTPUT_COMPLIANCE 0
#define MG_OUTPUT_MEAN_TEMPERATURE 1
int mg_output_derivative(mg_problem *p, int32_t output, const double *X, double *dq_dX);
/* One element at an element-local solution: the per-element plugin call
   MAST::NonlinearImplicitAssemblyElemOperations::elem_calculations(if_jac, vec, mat)
   after init(elem) and set_elem_solution(sol)
   (src/base/nonlinear_implicit_assembly_elem_operations.h:50-60,
   src/base/assembly_elem_operation.h:94-139; structural_nonlinear_assembly.cpp:112-139).
   sol_elem, fe: npe*dpn values, Ke: (npe*dpn)^2 row-major, all var-blocked (component c
   of local node a at c*npe + a).  fe = f_int - f_ext of the element's own loads (heat
   convection and source, side loads); point loads are the assembly's.  Ke or fe nullable. */
int mg_element_calculations(mg_problem *p, int64_t elem, const double *sol_elem, double *Ke,
                            double *fe);
/* d fe / dp for one parameter (kind, index as mg_sensitivity_assemble) at the element-local
   solution: NonlinearImplicitAssemblyElemOperations::elem_sensitivity_calculations
   (src/base/nonlinear_implicit_assembly_elem_operations.h:75-80,
   structural_nonlinear_assembly.cpp:170-196).  Zero for another element's parameter. */
int mg_element_sensitivity(mg_problem *p, int64_t elem, const double *sol_elem, int32_t kind,
                           int64_t index, double *dfe);
int mg_mean_temperature(mg_problem *p, const double *T, const mg_solve_opts *opts,
                        double *qbar, double *dq_dk0, double *dq_ds);

/* ---- testing hook ---- */
/* Host-side fault injection: the countdown-th next device allocation made by
   the library reports MG_ENOMEM (-1 disables).  No GPU fault is involved. */
void mg_debug_fail_alloc_after(int countdown);
/* One application of the mixed-precision matrix-free operator y = A x
   (precision MG_MIXED_TF32 / MG_MIXED_BF16 / MG_MIXED_TF32X3 / MG_MIXED_BF16X3: the
   tensor-core operator; MG_OPERATOR_FACTORED_FP32: the factored FP32 CUDA-core
   operator of the multigrid levels; x must be zero on Dirichlet dofs). */
#define MG_OPERATOR_FACTORED_FP32 100
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
   (MG_PLAIN_FP64) or the tensor-core column operator (MG_MIXED_*). */
int mg_debug_launch_apply(mg_problem *p, int precision, int reps);
/* Enqueues `reps` assemblies (residual and tangent, every colour) of the nonlinear-strain
   HEX8 element at X without synchronising; X (host, nullable) is copied first, NULL reuses
   the previously copied state.  MG_ENOTSUP for other physics. */
int mg_debug_launch_assembly(mg_problem *p, const double *X, int reps);

/* ---- allocation-free solve ---- */
/* No counterpart in the reference (MAST hands its linear systems to PETSc).
   Jacobi-preconditioned CG on a caller-owned CSR (n rows, int32 rowptr/cols,
   FP64 values, all device pointers) with right-hand side b and initial guess /
   solution x (device pointers), to ||b - A x|| <= rtol ||b||, enqueued on
   `stream` (a cudaStream_t; NULL = default stream).  It is for callers that
   cannot call cudaMalloc: code that must not allocate after start-up (a
   request loop running inside a fixed device-memory budget) and host
   applications whose own pool owns all device memory.  The library allocates
   nothing here: its scratch is one static device array of about 5.3 MB that
   every GPU loading the library holds until exit, which limits n to
   MG_STATIC_PCG_MAX_N (larger n returns MG_EINVAL).  Each call looks the
   array's address up in the current device's context (cudaGetSymbolAddress).
   The call blocks the calling thread until the solve ends: it synchronises
   `stream` every 16 iterations to read the convergence state, so it must not be
   called while `stream` is being captured into a graph.  All calls share
   the array, so calls that overlap on the GPU race; serialise them.  Returns
   MG_OK, MG_ENOCONV, MG_EBREAKDOWN or MG_ENAN; *iterations and *relres
   (nullable) report the iteration count and final relative residual. */
#define MG_STATIC_PCG_MAX_N 131072
int mg_pcg_csr_static(int64_t n, const int32_t *rowptr, const int32_t *cols, const double *vals,
                      const double *b, double *x, double rtol, int32_t max_iterations,
                      void *stream, int32_t *iterations, double *relres);

/* ---- batched design evaluations ----
   No single counterpart in the reference: MAST evaluates one design at a time
   (examples/structural/example_6/example_6.cpp:450-655 `evaluate`: set the
   density field, NonlinearSystem::solve, ComplianceOutput and
   calculate_output_adjoint_sensitivity_multiple_parameters_no_direct).  A batch
   holds many such SIMP cantilever evaluations of uneven structured-grid sizes,
   each with 1..MG_BATCH_MAX_CASES load cases sharing the design's stiffness, and
   solves all of them together with the mixed-precision matrix-free form
   (multi-problem persistent kernels driven by per-problem offset tables,
   graph-captured CG iterations, FP64 refinement).  Every load case is one
   problem; problems are numbered design by design, case by case. */
#define MG_BATCH_MAX_CASES 8

typedef struct mg_batch mg_batch;

typedef struct mg_batch_problem {
    int32_t nx, ny, nz;       /* unit-spaced HEX8 grid (libMesh build_cube numbering) */
    int32_t n_cases;          /* load cases, 1..MG_BATCH_MAX_CASES */
    const double *rho;        /* nx*ny*nz element densities in [0,1], x fastest */
    const int32_t *span;      /* 2*n_cases: node range [j0, j1] (inclusive) of a unit -z line
                                 load spread evenly over the nodes (nx, j, 0), j0 <= j <= j1;
                                 nullable when F is given */
    const double *F;          /* n_cases x 3*(nx+1)*(ny+1)*(nz+1) nodal loads, node-interleaved
                                 (overrides span; nullable) */
    const uint8_t *node_fix;  /* per node: bit c set = component c fixed; nullable: the x = 0
                                 face clamped */
} mg_batch_problem;

int mg_batch_create(const mg_batch_problem *designs, int32_t n_designs,
                    const mg_material_desc *mat, mg_batch **out);
void mg_batch_destroy(mg_batch *b);
/* totals: designs, problems (load cases), level-0 dofs, multigrid levels, device bytes */
int mg_batch_info(const mg_batch *b, int32_t *n_designs, int32_t *n_problems, int64_t *n_dofs,
                  int32_t *n_levels, int64_t *device_bytes);
void *mg_batch_stream(mg_batch *b);
/* replace design d's densities (host or device pointer); its solutions stay
   resident as the next warm start */
int mg_batch_set_design(mg_batch *b, int32_t d, const double *rho);
int mg_batch_set_design_device(mg_batch *b, int32_t d, const double *rho_device);
/* Solve every problem (opts->precision must be a mixed form; opts->warm_start
   starts from the resident solutions), then form compliance f.u and dC/drho for
   every problem.  reports (nullable) receives one entry per problem.  Returns
   MG_OK or the first failing problem's status. */
int mg_batch_solve(mg_batch *b, const mg_solve_opts *opts, mg_solve_report *reports);
/* the same restricted to the problems with active[i] != 0; the others keep
   their solutions and results */
int mg_batch_solve_subset(mg_batch *b, const mg_solve_opts *opts, const uint8_t *active,
                          mg_solve_report *reports);
/* design d's results (each nullable): compliance[n_cases], dc[n_cases * n_elems],
   u[n_cases * n_dofs] (node-interleaved) */
int mg_batch_results(mg_batch *b, int32_t d, double *compliance, double *dc, double *u);
/* Autotuner: times trial solves of one design per distinct grid shape over the
   solver-schedule knobs (precision within the family of opts->precision, smoother
   and coarse Chebyshev degrees, CG iterations per graph, inner tolerance, vector
   kernel grid), keeps the fastest that converges, writes it into *opts and caches
   it per shape set in the process (and in the file named by MG_TUNE_CACHE when
   that is set).  A cache hit runs no trial.  *seconds (nullable) gets the best
   trial time. */
int mg_batch_autotune(mg_batch *b, mg_solve_opts *opts, int32_t max_trials, double *seconds);

/* ---- request loop (continuous batching of design evaluations) ----
   No counterpart in the reference (its design loop calls `evaluate` serially,
   examples/structural/example_6/example_6.cpp:450-655).  A server owns a worker
   thread and the resident chains, held in a few shards (batches with a stream
   each, stepped on the GPU together).  Requests belong to design chains: a chain has one
   grid and one number of load cases; its mesh tables and last solutions stay
   resident in device memory and every request of the chain warm-starts from the
   chain's previous solution.  Requests that arrive while others are on the GPU
   join the running multi-problem solve at the next step boundary (a few CG
   iterations), so work of different requests overlaps in the same kernels.  New
   chains are admitted against the device-memory cap without stopping the
   resident ones (a shard of their own, or an idle shard rebuilt with them); only
   when the cap requires evictions (least recently used idle chains first) does
   the worker let the in-flight work finish and rebuild; a chain that cannot fit
   alone is rejected (MG_ENOMEM in its completions). */
typedef struct mg_server mg_server;

typedef struct mg_request {
    int32_t chain;            /* design chain id, >= 0 */
    int32_t nx, ny, nz;       /* the chain's grid (fixed per chain) */
    int32_t n_cases;          /* the chain's load cases (fixed per chain) */
    int32_t reserved;
    const double *rho;        /* nx*ny*nz densities in [0,1]; copied by mg_server_submit */
    const int32_t *span;      /* 2*n_cases unit -z line-load node spans (as mg_batch_problem);
                                 copied by mg_server_submit */
    double *compliance_out;   /* n_cases, caller-owned, filled before the completion is posted
                                 (nullable) */
    double *dc_out;           /* n_cases * nx*ny*nz dC/drho, caller-owned (nullable) */
    double arrival_s;         /* arrival time on the mg_server_clock() scale (<= 0: now) */
    uint64_t tag;             /* echoed in the completion */
} mg_request;

typedef struct mg_completion {
    uint64_t tag;
    int32_t chain, status;
    int32_t krylov_iterations, refinements; /* summed / maximum over the request's load cases */
    double relres;                          /* maximum FP64 relative residual over the cases */
    double arrival_s, admit_s, done_s;      /* mg_server_clock() times */
} mg_completion;

typedef struct mg_server_opts {
    int64_t hbm_cap_bytes;    /* cap on the resident tables of all chains (0 = 150 GB) */
    mg_solve_opts solve;      /* mixed-precision form, tolerances, warm starts implied */
    int32_t max_inflight;     /* designs on the GPU at once (0 = no limit) */
    int32_t reserved;
} mg_server_opts;

typedef struct mg_server_stats {
    int64_t submitted, completed, failed, rebuilds, evictions;
    int64_t resident_bytes, peak_resident_bytes;
    int32_t resident_chains, inflight, peak_inflight, reserved;
    double p50_s, p99_s, mean_s, max_s;   /* latency: arrival -> results posted */
    double solves_per_s;                  /* completed requests / (last completion - first arrival) */
    double dofs_per_s;                    /* solved dofs (all load cases) per second */
} mg_server_stats;

double mg_server_clock(void);
int mg_server_create(const mg_material_desc *mat, const mg_server_opts *opts, mg_server **out);
/* thread-safe; MG_EINVAL for a malformed request or one that contradicts its chain */
int mg_server_submit(mg_server *s, const mg_request *req);
/* up to max completions posted since the last poll, waiting up to timeout_s for the first */
int mg_server_poll(mg_server *s, mg_completion *out, int32_t max, int32_t *n, double timeout_s);
/* wait until every submitted request has completed (MG_ETIMEDOUT after timeout_s > 0) */
int mg_server_drain(mg_server *s, double timeout_s);
int mg_server_get_stats(mg_server *s, mg_server_stats *out);
/* stops the worker after the submitted requests complete, frees everything */
void mg_server_destroy(mg_server *s);

/* Synthetic request stream for benchmarks: n_requests Poisson arrivals at `rate`
   req/s over n_chains chains; chain grids drawn uniformly from sizes (3 ints
   each), except round(big_fraction * n_chains) chains (at least one when
   big_fraction > 0) on the big grid; 1..max_cases load cases per chain with
   seeded spans; densities start iid U[0.01,1] and each request adds N(0, noise)
   clipped to [0.01, 1].  All densities are generated before the clock starts;
   a submitter thread then submits each request at its arrival time and the call
   returns after the last completion with the server statistics of this run.
   compliance_out (nullable): n_requests x max_cases (unused cases 0). */
typedef struct mg_synthetic_desc {
    int64_t n_requests;
    double rate;
    int32_t n_chains, n_sizes;
    const int32_t *sizes;
    double big_fraction;
    int32_t big_nx, big_ny, big_nz, max_cases;
    double noise;
    uint64_t seed;
} mg_synthetic_desc;
int mg_server_run_synthetic(mg_server *s, const mg_synthetic_desc *desc, double *compliance_out,
                            mg_server_stats *stats);
/* Request `index` of the synthetic stream `desc` describes, regenerated from the same
   seeded generator (no server needed): info[5] = chain, nx, ny, nz, n_cases; span
   (nullable) 2*n_cases load spans; rho (nullable) nx*ny*nz densities, bitwise those that
   mg_server_run_synthetic submitted for that request.  For checking served results
   against an independent solve. */
int mg_server_synthetic_request(const mg_synthetic_desc *desc, int64_t index, int32_t *info,
                                int32_t *span, double *rho);

/* ---- density filter ----
   MAST::FilterBase (src/level_set/filter_base.cpp): x_filtered_i =
   sum_j w_ij x_j over the points j within `radius` of point i, w_ij = (radius -
   d_ij) / sum_k (radius - d_ik) (`_init` :378-437, `_init2` :275-359); points
   not flagged in dv_mask keep their value (compute_filtered_values :58-95).
   transpose = 1 applies F^T: the chain rule of a design gradient taken with
   respect to the filtered field (examples/structural/example_6/example_6.cpp:661-697). */
typedef struct mg_filter mg_filter;
/* element centroids of a structured grid with spacings hx, hy, hz (nz = 0: 2D
   grid); dv_mask nullable (every element is a design variable) */
int mg_filter_create_grid(int32_t nx, int32_t ny, int32_t nz, double hx, double hy, double hz,
                          double radius, const uint8_t *dv_mask, mg_filter **out);
/* arbitrary points (n x dim coordinates, dim 1..3) */
int mg_filter_create_points(int64_t n, int32_t dim, const double *xyz, double radius,
                            const uint8_t *dv_mask, mg_filter **out);
int mg_filter_info(const mg_filter *f, int64_t *n, int64_t *nnz);
int mg_filter_apply(mg_filter *f, const double *in, double *out, int32_t transpose);
/* device pointers (in != out), on `stream` (NULL: the filter's own stream; no sync) */
int mg_filter_apply_device(mg_filter *f, const double *in_dev, double *out_dev, int32_t transpose,
                           void *stream);
void mg_filter_destroy(mg_filter *f);

/* ---- Nastran bulk data (BDF) mesh input ----
   Replaces MAST::NastranIO::read (src/mesh/nastran_io.cpp:221-339; read_nodes
   :105-125, read_elements :128-198, read_node_boundaries :201-218), which reads
   through pyNastran.  Host code, no GPU.  Small-field, large-field (NAME*) and
   free-field cards with continuation lines; GRID (basic coordinates), CHEXA
   (8 nodes), CQUAD4, SPC1 (with THRU), SPC (D = 0) and FORCE (basic
   coordinates).  Nodes in ascending GRID id, elements in ascending element id,
   element nodes in the card's order (libMesh's local order); constraints and
   loads of every set id.  The arrays feed mg_mesh_desc / mg_bc_desc. */
/* ---- ExodusII files (host only) ----
   MAST writes its solutions through libMesh's ExodusII_IO
   (examples/structural/example_7/example_7.cpp:256-281: write_timestep of the
   mesh, nodal and element variables).  mg_exodus_write writes one time step of a
   HEX8 (nodes_per_elem 8, dim 3) or QUAD4 (4, dim 2 or 3) mesh in the netCDF
   classic format with 64-bit offsets: coordinates (n_nodes x dim), one element
   block (0-based conn, written 1-based), n_nodal_vars nodal fields
   (n_nodal_vars x n_nodes, e.g. displacement components) and n_elem_vars element
   fields (n_elem_vars x n_elems, e.g. density, dC/drho).  mg_exodus_read_sizes /
   mg_exodus_read_mesh read the mesh of a netCDF classic (CDF-1 or CDF-2) ExodusII
   file: coordinates and the connectivity of every element block (one element
   type), 0-based.  netCDF-4 / HDF5 files are not read (MG_EINVAL). */
int mg_exodus_write(const char *path, const char *title, int32_t dim, int32_t nodes_per_elem, int64_t n_nodes,
                    const double *coords, int64_t n_elems, const int32_t *conn, int32_t n_nodal_vars,
                    const char *const *nodal_names, const double *nodal_vals, int32_t n_elem_vars,
                    const char *const *elem_names, const double *elem_vals, double time);
int mg_exodus_read_sizes(const char *path, int32_t *dim, int32_t *nodes_per_elem, int64_t *n_nodes,
                         int64_t *n_elems);
int mg_exodus_read_mesh(const char *path, double *coords, int32_t *conn);

typedef struct mg_bdf_mesh mg_bdf_mesh;
int mg_bdf_read(const char *path, mg_bdf_mesh **out);
int mg_bdf_parse(const char *text, int64_t len, mg_bdf_mesh **out);
int mg_bdf_sizes(const mg_bdf_mesh *m, int64_t *n_nodes, int64_t *n_elems, int32_t *nodes_per_elem);
/* coords: n_nodes x 3; grid_ids (nullable): the GRID id of each node */
int mg_bdf_nodes(const mg_bdf_mesh *m, double *coords, int64_t *grid_ids);
/* conn: n_elems x nodes_per_elem node indices; elem_ids, pids nullable */
int mg_bdf_elements(const mg_bdf_mesh *m, int32_t *conn, int64_t *elem_ids, int32_t *pids);
/* homogeneous Dirichlet dofs (dof = dpn*node + component - 1, components
   1..dpn of the SPC digits); fixed_dofs NULL: only *n */
int mg_bdf_constraints(const mg_bdf_mesh *m, int32_t dpn, int64_t *fixed_dofs, int64_t *n);
/* nodal point loads F (components 1..min(dpn, 3)), summed per dof; NULL arrays: only *n */
int mg_bdf_loads(const mg_bdf_mesh *m, int32_t dpn, int64_t *load_dofs, double *load_values, int64_t *n);
void mg_bdf_destroy(mg_bdf_mesh *m);

/* parameter kinds for mg_sensitivity_assemble */
#define MG_PARAM_DENSITY 0      /* rho_e of element param_index (elasticity) */
#define MG_PARAM_K0 1           /* conductivity k0 (heat) */
#define MG_PARAM_ELEM_SCALE 2   /* conductivity scale s_e of element param_index (heat) */

#ifdef __cplusplus
}
#endif
#endif /* MASTGPU_H */
