// batch.h -- internal state of a batch of SIMP design evaluations (mg_batch),
// shared by the batch entry points and the request loop.
#pragma once

#include <vector>

#include "matfree.cuh"

struct mg_batch {
    cudaStream_t stream = nullptr;
    mg_material_desc mat{};
    int n_designs = 0, n_probs = 0;
    std::vector<int> nx, ny, nz, cases, first;  // per design; first = its case-0 problem
    std::vector<int> design_of;                 // per problem
    std::vector<int64_t> rho_off;               // per design: offset of its densities
    std::vector<int64_t> dc_off;                // per problem: offset of its dC/drho
    int64_t n_rho = 0, n_dc = 0, max_dofs = 0;
    mg::MfBatch mf;
    double *d_rho = nullptr, *d_E = nullptr, *d_dE = nullptr, *d_dc = nullptr, *d_u = nullptr;
    int *d_status = nullptr;
    std::vector<double> compliance;             // per problem
    std::vector<mg_solve_report> reports;       // per problem, last solve
    int64_t device_bytes = 0;
};

namespace mg {

inline int64_t dofs_of(int nx, int ny, int nz) { return 3LL * (nx + 1) * (ny + 1) * (nz + 1); }
bool material_ok(const mg_material_desc &m);
// unit -z line load spread evenly over the nodes (nx, j, 0), j0 <= j <= j1
void line_load(int nx, int ny, int nz, int j0, int j1, std::vector<double> &F);
// per-node Dirichlet bits of the clamped x = 0 face
void clamp_x0(int nx, int ny, int nz, std::vector<uint8_t> &fix);
int read_device_status(mg_batch *b);
// E(rho), dE/drho of design d from the resident densities, into the batch tables
int refresh_moduli(mg_batch *b, int d);
int64_t batch_bytes(const MfBatch &m);
MfSolveParams params_from(const mg_solve_opts &o);
// solve (a subset of) the batch, then compliance and sensitivities of the solved problems
int batch_solve(mg_batch *b, const mg_solve_opts &o, const uint8_t *active, mg_solve_report *reports);
// compliance and dc of the problems in `active` from their resident solutions
int batch_results_of(mg_batch *b, const uint8_t *active);

}  // namespace mg
