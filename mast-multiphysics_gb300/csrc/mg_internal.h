// mg_internal.h -- shared declarations of the CUDA hot path behind mastgpu.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mastgpu.h"

namespace mg {

void set_error(const char *fmt, ...);

#define MG_CUDA_TRY(expr)                                                        \
    do {                                                                         \
        cudaError_t _e = (expr);                                                 \
        if (_e != cudaSuccess) {                                                 \
            ::mg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,           \
                            cudaGetErrorString(_e));                             \
            return _e == cudaErrorMemoryAllocation ? MG_ENOMEM : MG_ECUDA;       \
        }                                                                        \
    } while (0)

#define MG_TRY(expr)                 \
    do {                             \
        int _s = (expr);             \
        if (_s != MG_OK) return _s;  \
    } while (0)

// Device allocation with a host-side failure-injection hook (tests set the
// countdown; when it reaches zero the next allocation reports MG_ENOMEM).
int dev_alloc(void **ptr, size_t bytes);
void dev_free(void *ptr);
template <class T>
int dev_alloc_n(T **ptr, size_t n) {
    return dev_alloc(reinterpret_cast<void **>(ptr), n * sizeof(T));
}

// Krylov solver state resident in device memory.  All scalars are produced by
// deterministic last-block reductions and read by the next kernel.
struct KrylovState {
    double rz, rz_new, rr, pq, alpha, beta, omega, rho, bb, tol2;
    double ts, tt, rv;
    int iter, done, status, maxit;
    unsigned int counter;
    int pad;
};

// Scratch used by the Krylov kernels (one set per problem).
struct KrylovWork {
    int64_t n = 0;
    int grid = 0;            // blocks of the vector kernels (fixed: deterministic sums)
    double *r = nullptr, *z = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr;
    double *dinv = nullptr;
    double *rh = nullptr, *v = nullptr, *y = nullptr, *s = nullptr, *t = nullptr;
    double *partials = nullptr; // 3 * grid
    KrylovState *state = nullptr;
    KrylovState *state_host = nullptr; // pinned mirror
    cudaGraphExec_t graph_cg[2] = {nullptr, nullptr};
    int graph_chunk = 0;
    cudaGraphExec_t graph_bicg = nullptr;
    int bicg_chunk = 0;
};

struct CsrMatrix {
    int64_t n = 0, nnz = 0;
    int dpn = 1;
    int32_t *rowptr = nullptr, *cols = nullptr;
    double *vals = nullptr;
};

struct MatfreeWork;  // mixed-precision matrix-free state (matfree.cu)

}  // namespace mg

struct mg_problem {
    int physics = 0, dim = 3, npe = 8, dpn = 3;
    int64_t n_nodes = 0, n_elems = 0, n_dofs = 0;
    int grid_nx = 0, grid_ny = 0, grid_nz = 0;
    mg_material_desc mat{};
    cudaStream_t stream = nullptr;
    int device = 0;

    // host copies of the set-up tables
    std::vector<double> h_coords;
    std::vector<int32_t> h_conn;
    std::vector<uint8_t> h_fixed;
    std::vector<double> h_F;         // external load: point loads + side loads
    std::vector<double> h_F_point;   // the point loads alone
    std::vector<int64_t> color_ptr;  // n_colors + 1 offsets into d_color_elems
    int n_colors = 0;

    // device mesh / property tables
    double *d_coords = nullptr;
    int32_t *d_conn = nullptr;
    int32_t *d_color_elems = nullptr;
    uint8_t *d_fixed = nullptr;
    double *d_F = nullptr;
    double *d_rho = nullptr, *d_E = nullptr, *d_dE = nullptr;
    // nodal density field (MeshFieldFunction over FIRST-order LAGRANGE): the
    // modulus and dE/drho at each Gauss point (n_elems x 8), the node -> (element,
    // corner) incidences 8 e + a in element order, scratch of the sensitivity
    bool nodal_design = false;
    double *d_rho_nodes = nullptr, *d_Eq = nullptr, *d_dEq = nullptr, *d_qp_out = nullptr,
           *d_node_out = nullptr;
    int32_t *d_node_inc_ptr = nullptr, *d_node_inc = nullptr;
    double *d_s = nullptr, *d_q = nullptr;
    uint8_t *d_conv_mask = nullptr;  // per element bit mask of convection sides
    double conv_h = 0, conv_Tinf = 0;
    int64_t n_conv = 0;

    // CSR system and element -> CSR position map
    mg::CsrMatrix A;
    uint16_t *d_emap = nullptr;       // n_elems * npe * npe column-block offsets
    int64_t *d_fix_zero = nullptr;    // CSR positions zeroed by the Dirichlet elimination
    int64_t *d_fix_diag = nullptr;    // CSR diagonal positions of fixed rows
    int64_t n_fix_zero = 0, n_fix_diag = 0;
    bool jacobian_valid = false;
    bool last_solve_mixed = false;

    // state vectors
    double *d_X = nullptr, *d_R = nullptr, *d_tmp = nullptr, *d_tmp2 = nullptr;
    double *d_elem_out = nullptr;     // per-element scalar outputs
    double *d_ks = nullptr;           // KS stress output scratch (6 n_elems + 8), allocated on use
    double *d_side = nullptr;         // side-load values, n_elems x (6 HEX8 faces | 4 QUAD4 edges)
    double *d_red = nullptr;          // reduction scratch
    int red_blocks = 0;
    mg::KrylovWork kw;
    mg::MatfreeWork *mf = nullptr;
};

namespace mg {

// ---- assembly.cu ----
int assemble_system(mg_problem *p, const double *d_X, double *d_R, bool want_jacobian,
                    bool consistent);
int element_matrices(mg_problem *p, const double *d_X, int64_t first, int64_t count,
                     double *d_Ke, double *d_fe);
int launch_assembly(mg_problem *p, const double *d_X, int reps);
int assemble_side_loads(mg_problem *p);
// KS stress output (d_ks: 6 n_elems + 8 doubles of scratch)
int ks_stress_values(mg_problem *p, const double *d_X, double p_ks, double sigma0, double penal,
                     double *d_ks, double host_out[3]);
int ks_stress_gradient(mg_problem *p, const double *d_X, double p_ks, double sigma0,
                       const double *d_ks, double scale, double *d_g);
int ks_stress_combine(mg_problem *p, const double *d_ks, double inv_s0I, const double *d_adj,
                      double *d_out);
int compute_modulus(mg_problem *p);
// SIMP E(rho), dE/drho of n elements on stream s; bit 4 of *d_status marks a
// density outside [0,1] or NaN
int compute_nodal_modulus(mg_problem *p);
int nodal_compliance_sensitivity(mg_problem *p, const double *d_u, double *dc_dev);
int launch_simp_modulus(const double *d_rho, int64_t n, const mg_material_desc &mat, double *d_E,
                        double *d_dE, int *d_status, cudaStream_t s);
int build_emap(mg_problem *p);
int elem_sensitivity(mg_problem *p, const double *d_X, const double *d_lambda, int kind,
                     double *d_out_elem);
int assemble_param_residual(mg_problem *p, const double *d_X, int kind, int64_t index,
                            double *d_dRdp);
int mean_temperature_terms(mg_problem *p, const double *d_T, double *d_dqdT, double *qbar);
// one element at an element-local solution (device pointers; d_elem_slot: one device int32)
int element_calculations(mg_problem *p, int64_t e, const double *d_sol, double *d_Ke,
                         double *d_fe, int32_t *d_elem_slot);
int element_sensitivity(mg_problem *p, int64_t e, const double *d_sol, int kind, int64_t index,
                        double *d_dfe);

// ---- krylov.cu ----
int krylov_init(mg_problem *p);
void krylov_free(mg_problem *p);
int spmv(mg_problem *p, const CsrMatrix &A, const double *d_x, double *d_y);
int krylov_solve(mg_problem *p, const CsrMatrix &A, const double *d_b, double *d_x,
                 const mg_solve_opts &o, int krylov, int *iters, double *relres);
int dot(mg_problem *p, const double *a, const double *b, int64_t n, double *out);
int transpose_csr(mg_problem *p, const CsrMatrix &A, CsrMatrix *At);
void free_csr(CsrMatrix *A);

// ---- matfree.cu ----
// x_zero: the initial guess is 0 (the first refinement residual is f, no operator pass)
int matfree_solve(mg_problem *p, const mg_solve_opts &o, mg_solve_report *rep, bool x_zero);
int matfree_apply_debug(mg_problem *p, int precision, const double *x_host, double *y_host);
int matfree_sensitivity(mg_problem *p, double *dc_host);
int matfree_compliance_resident(mg_problem *p, double *compliance);
int matfree_launch_apply(mg_problem *p, int precision, int reps);
int krylov_launch_spmv_cg(mg_problem *p, int reps);
void matfree_free(mg_problem *p);

double wall_time();

// number of kernel launches issued by this library (graph nodes included)
void count_launches(long long n);

}  // namespace mg
