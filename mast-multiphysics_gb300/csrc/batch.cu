// batch.cu -- batched SIMP design evaluations (mg_batch_*) on the multi-problem
// matrix-free solver, and the autotuner of its solver schedule.
//
// A design is one structured-grid SIMP cantilever with 1..MG_BATCH_MAX_CASES
// load cases.  Every load case is one level-0 problem of the MfBatch; the cases
// of a design share its element moduli (MfProblem::share_elems) and so its
// multigrid coarse-level moduli.  The reference evaluates one design per call
// (examples/structural/example_6/example_6.cpp:450-655: set the density field,
// NonlinearSystem::solve, ComplianceOutput, adjoint sensitivities); here all
// designs advance together through the same persistent kernels.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "batch.h"

namespace mg {

bool material_ok(const mg_material_desc &m) {
    return m.E0 > 0.0 && m.Emin >= 0.0 && m.Emin < m.E0 && m.nu > -1.0 && m.nu < 0.5 &&
           m.penal >= 1.0 && isfinite(m.E0) && isfinite(m.penal);
}

// unit -z line load spread evenly over the nodes (nx, j, 0), j0 <= j <= j1
void line_load(int nx, int ny, int nz, int j0, int j1, std::vector<double> &F) {
    const int NX = nx + 1, NY = ny + 1;
    F.assign((size_t)dofs_of(nx, ny, nz), 0.0);
    const double v = -1.0 / (double)(j1 - j0 + 1);
    for (int j = j0; j <= j1; j++) F[3 * ((size_t)nx + (size_t)NX * j) + 2] = v;
    (void)NY;
}

// per-node Dirichlet bits of the clamped x = 0 face
void clamp_x0(int nx, int ny, int nz, std::vector<uint8_t> &fix) {
    const size_t NX = nx + 1, NY = ny + 1, NZ = nz + 1;
    fix.assign(NX * NY * NZ, 0);
    for (size_t k = 0; k < NZ; k++)
        for (size_t j = 0; j < NY; j++) fix[NX * (j + NY * k)] = 7;
}

int read_device_status(mg_batch *b) {
    int h = 0;
    MG_CUDA_TRY(cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    if (h & 4) {
        set_error("design density outside [0,1] or NaN");
        return MG_EINVAL;
    }
    return MG_OK;
}

// E(rho), dE/drho of design d from the resident densities, into the batch tables
int refresh_moduli(mg_batch *b, int d) {
    const int64_t ne = (int64_t)b->nx[d] * b->ny[d] * b->nz[d];
    MG_TRY(launch_simp_modulus(b->d_rho + b->rho_off[d], ne, b->mat, b->d_E + b->rho_off[d],
                               b->d_dE + b->rho_off[d], b->d_status, b->stream));
    return mf_batch_set_moduli(b->mf, b->first[d], b->d_E + b->rho_off[d], b->d_dE + b->rho_off[d]);
}

int64_t batch_bytes(const MfBatch &m) {
    const int64_t f32_vecs = 13, f64_vecs = 3;
    return m.n_pad * (4 * f32_vecs + 8 * f64_vecs) + m.n_elem_pad * 20 + m.n_nodes +
           (int64_t)m.n_probs * (sizeof(MfProblem) + sizeof(MfState) + kMapsPerProblem * 128) +
           (int64_t)m.n_bricks * (sizeof(MfBrick) + 16) + (int64_t)m.n_chunks * (sizeof(MfChunkDesc) + 16);
}

MfSolveParams params_from(const mg_solve_opts &o) {
    MfSolveParams prm;
    prm.precision = o.precision;
    prm.rtol = o.rtol > 0 ? o.rtol : 1e-8;
    prm.inner_rtol = o.inner_rtol > 0 ? o.inner_rtol : 1e-3;
    prm.max_iterations = o.max_iterations;
    prm.max_refinements = o.max_refinements;
    prm.graph_chunk = o.graph_chunk;
    prm.timeout_s = o.timeout_s;
    prm.mg = (o.preconditioner == MG_PC_MULTIGRID) ? 1 : 0;
    prm.smooth_deg = o.smooth_degree;
    prm.coarse_deg = o.coarse_degree;
    prm.vec_blocks_per_sm = o.vec_blocks_per_sm;
    prm.mg_operator = o.smoother_operator == MG_SMOOTHER_TENSOR ? 1 : 0;
    prm.active = nullptr;
    return prm;
}

// solve (a subset of) the batch, then compliance and sensitivities of the
// solved problems
int batch_solve(mg_batch *b, const mg_solve_opts &o, const uint8_t *active, mg_solve_report *reports) {
    if (o.precision < MG_MIXED_TF32 || o.precision > MG_MIXED_BF16X3) {
        set_error("batched solves use the mixed-precision forms (precision %d)", o.precision);
        return MG_ENOTSUP;
    }
    const double t0 = wall_time();
    MfSolveParams prm = params_from(o);
    prm.active = active;
    const int rc = mf_batch_solve(b->mf, prm, o.warm_start != 0);
    if (rc == MG_ETIMEDOUT || rc == MG_ECUDA || rc == MG_ENOMEM) return rc;
    MG_TRY(batch_results_of(b, active));
    const double secs = wall_time() - t0;
    for (int i = 0; i < b->n_probs; i++) {
        if (active && !active[i]) continue;
        b->reports[i].seconds = secs;
        if (reports) reports[i] = b->reports[i];
    }
    return rc;
}

int batch_results_of(mg_batch *b, const uint8_t *active) {
    std::vector<double> comp(b->n_probs, 0.0);
    MG_TRY(mf_batch_compliance(b->mf, comp.data(), b->d_dc, active));
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < b->n_probs; i++) {
        if (active && !active[i]) continue;
        b->compliance[i] = comp[i];
        const MfState &h = b->mf.states_host[i];
        mg_solve_report &r = b->reports[i];
        r.status = h.ref_status;
        r.newton_iterations = 1;
        r.krylov_iterations = h.total_iter;
        r.refinements = h.refine;
        r.relres = h.ff64 > 0.0 ? sqrt(h.rr64 / h.ff64) : 0.0;
        r.residual_norm = sqrt(h.rr64);
        r.seconds = 0.0;
    }
    return MG_OK;
}

namespace {

// ------------------------------------------------------------------ autotuner
struct TuneEntry {
    int precision, smooth, coarse, chunk, vec_blocks;
    double inner_rtol, seconds;
    int smoother = MG_SMOOTHER_FACTORED;
};

std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune_cache;
bool g_tune_file_loaded = false;

std::string tune_key(const mg_batch *b, const mg_solve_opts &o) {
    std::vector<std::string> shapes;
    for (int d = 0; d < b->n_designs; d++) {
        char s[64];
        snprintf(s, sizeof(s), "%dx%dx%d", b->nx[d], b->ny[d], b->nz[d]);
        shapes.push_back(s);
    }
    std::sort(shapes.begin(), shapes.end());
    shapes.erase(std::unique(shapes.begin(), shapes.end()), shapes.end());
    const bool bf16 = (o.precision == MG_MIXED_BF16 || o.precision == MG_MIXED_BF16X3);
    char head[96];
    snprintf(head, sizeof(head), "%s|pc%d|rtol%.0e|", bf16 ? "bf16" : "tf32", o.preconditioner, o.rtol);
    std::string k = head;
    for (auto &s : shapes) k += s + ",";
    return k;
}

void tune_file_load() {
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const char *path = getenv("MG_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char key[4096];
    TuneEntry e;
    while (fscanf(f, "%4095s %d %d %d %d %d %lf %lf %d", key, &e.precision, &e.smooth, &e.coarse,
                  &e.chunk, &e.vec_blocks, &e.inner_rtol, &e.seconds, &e.smoother) == 9)
        g_tune_cache[key] = e;
    fclose(f);
}

void tune_file_save() {
    const char *path = getenv("MG_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "w");
    if (!f) return;
    for (auto &kv : g_tune_cache)
        fprintf(f, "%s %d %d %d %d %d %.3e %.6e %d\n", kv.first.c_str(), kv.second.precision,
                kv.second.smooth, kv.second.coarse, kv.second.chunk, kv.second.vec_blocks,
                kv.second.inner_rtol, kv.second.seconds, kv.second.smoother);
    fclose(f);
}

void apply_entry(const TuneEntry &e, mg_solve_opts &o) {
    o.precision = e.precision;
    o.smooth_degree = e.smooth;
    o.coarse_degree = e.coarse;
    o.graph_chunk = e.chunk;
    o.vec_blocks_per_sm = e.vec_blocks;
    o.inner_rtol = e.inner_rtol;
    o.smoother_operator = e.smoother;
}

}  // namespace
}  // namespace mg

using namespace mg;

extern "C" {

int mg_batch_create(const mg_batch_problem *designs, int32_t n_designs, const mg_material_desc *mat,
                    mg_batch **out) {
    if (!out) return MG_EINVAL;
    *out = nullptr;
    if (!designs || n_designs <= 0 || !mat) {
        set_error("mg_batch_create: null argument or empty batch");
        return MG_EINVAL;
    }
    if (!material_ok(*mat)) {
        set_error("mg_batch_create: material out of range");
        return MG_EINVAL;
    }
    for (int d = 0; d < n_designs; d++) {
        const mg_batch_problem &p = designs[d];
        if (p.nx <= 0 || p.ny <= 0 || p.nz <= 0 || p.nx > 4096 || p.ny > 4096 || p.nz > 4096) {
            set_error("design %d: bad grid %dx%dx%d", d, p.nx, p.ny, p.nz);
            return MG_EINVAL;
        }
        if (p.n_cases < 1 || p.n_cases > MG_BATCH_MAX_CASES || !p.rho || (!p.span && !p.F)) {
            set_error("design %d: need 1..%d load cases, densities and loads", d, MG_BATCH_MAX_CASES);
            return MG_EINVAL;
        }
        const int64_t ne = (int64_t)p.nx * p.ny * p.nz;
        for (int64_t e = 0; e < ne; e++)
            if (!(p.rho[e] >= 0.0 && p.rho[e] <= 1.0)) {
                set_error("design %d: density %lld = %g outside [0,1]", d, (long long)e, p.rho[e]);
                return MG_EINVAL;
            }
        if (!p.F)
            for (int c = 0; c < p.n_cases; c++)
                if (p.span[2 * c] < 0 || p.span[2 * c] > p.span[2 * c + 1] || p.span[2 * c + 1] > p.ny) {
                    set_error("design %d case %d: load span [%d,%d] outside [0,%d]", d, c, p.span[2 * c],
                              p.span[2 * c + 1], p.ny);
                    return MG_EINVAL;
                }
    }
    mg_batch *b = new mg_batch();
    b->mat = *mat;
    b->n_designs = n_designs;
    auto fail = [&](int rc) {
        mg_batch_destroy(b);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        set_error("cudaStreamCreate failed (no usable GPU?)");
        return MG_ECUDA;
    }
    std::vector<MfProblem> shapes;
    for (int d = 0; d < n_designs; d++) {
        const mg_batch_problem &p = designs[d];
        b->nx.push_back(p.nx);
        b->ny.push_back(p.ny);
        b->nz.push_back(p.nz);
        b->cases.push_back(p.n_cases);
        b->first.push_back((int)shapes.size());
        b->rho_off.push_back(b->n_rho);
        b->n_rho += (int64_t)p.nx * p.ny * p.nz;
        b->max_dofs = std::max(b->max_dofs, dofs_of(p.nx, p.ny, p.nz));
        for (int c = 0; c < p.n_cases; c++) {
            MfProblem P{};
            P.nx = p.nx;
            P.ny = p.ny;
            P.nz = p.nz;
            P.share_elems = (c == 0) ? -1 : b->first[d];
            b->design_of.push_back(d);
            b->dc_off.push_back(b->n_dc);
            b->n_dc += (int64_t)p.nx * p.ny * p.nz;
            shapes.push_back(P);
        }
    }
    b->n_probs = (int)shapes.size();
    b->compliance.assign(b->n_probs, 0.0);
    b->reports.assign(b->n_probs, mg_solve_report{});
    int rc = mf_batch_init(b->mf, shapes, 1.0, 1.0, 1.0, mat->nu, b->stream);
    if (rc != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_rho, (size_t)b->n_rho)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_E, (size_t)b->n_rho)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_dE, (size_t)b->n_rho)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_dc, (size_t)b->n_dc)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_u, (size_t)b->max_dofs)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&b->d_status, 1)) != MG_OK) return fail(rc);
    b->device_bytes = batch_bytes(b->mf) + 8 * (3 * b->n_rho + b->n_dc + b->max_dofs);
    if (cudaMemsetAsync(b->d_status, 0, sizeof(int), b->stream) != cudaSuccess) return fail(MG_ECUDA);
    for (int d = 0; d < n_designs; d++) {
        const mg_batch_problem &p = designs[d];
        const int64_t ne = (int64_t)p.nx * p.ny * p.nz;
        if (cudaMemcpyAsync(b->d_rho + b->rho_off[d], p.rho, ne * 8, cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess)
            return fail(MG_ECUDA);
        if ((rc = refresh_moduli(b, d)) != MG_OK) return fail(rc);
        std::vector<uint8_t> fix;
        if (p.node_fix) fix.assign(p.node_fix, p.node_fix + (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1));
        else clamp_x0(p.nx, p.ny, p.nz, fix);
        std::vector<double> F;
        const int64_t nd = dofs_of(p.nx, p.ny, p.nz);
        for (int c = 0; c < p.n_cases; c++) {
            if (p.F) F.assign(p.F + c * nd, p.F + (c + 1) * nd);
            else line_load(p.nx, p.ny, p.nz, p.span[2 * c], p.span[2 * c + 1], F);
            if ((rc = mf_batch_set_bc(b->mf, b->first[d] + c, fix.data(), F.data())) != MG_OK) return fail(rc);
        }
        if ((rc = cudaStreamSynchronize(b->stream)) != cudaSuccess) return fail(MG_ECUDA);
    }
    if ((rc = read_device_status(b)) != MG_OK) return fail(rc);
    *out = b;
    return MG_OK;
}

void mg_batch_destroy(mg_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    mf_batch_free(b->mf);
    void *ptrs[] = {b->d_rho, b->d_E, b->d_dE, b->d_dc, b->d_u, b->d_status};
    for (void *q : ptrs) dev_free(q);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int mg_batch_info(const mg_batch *b, int32_t *n_designs, int32_t *n_problems, int64_t *n_dofs,
                  int32_t *n_levels, int64_t *device_bytes) {
    if (!b) return MG_EINVAL;
    if (n_designs) *n_designs = b->n_designs;
    if (n_problems) *n_problems = b->n_probs;
    if (n_dofs) {
        int64_t s = 0;
        for (int d = 0; d < b->n_designs; d++) s += b->cases[d] * dofs_of(b->nx[d], b->ny[d], b->nz[d]);
        *n_dofs = s;
    }
    if (n_levels) *n_levels = b->mf.n_levels;
    if (device_bytes) *device_bytes = b->device_bytes;
    return MG_OK;
}

void *mg_batch_stream(mg_batch *b) { return b ? (void *)b->stream : nullptr; }

int mg_batch_set_design(mg_batch *b, int32_t d, const double *rho) {
    if (!b || !rho || d < 0 || d >= b->n_designs) return MG_EINVAL;
    const int64_t ne = (int64_t)b->nx[d] * b->ny[d] * b->nz[d];
    for (int64_t e = 0; e < ne; e++)
        if (!(rho[e] >= 0.0 && rho[e] <= 1.0)) {
            set_error("density %lld = %g outside [0,1]", (long long)e, rho[e]);
            return MG_EINVAL;
        }
    MG_CUDA_TRY(cudaMemcpyAsync(b->d_rho + b->rho_off[d], rho, ne * 8, cudaMemcpyHostToDevice, b->stream));
    MG_TRY(refresh_moduli(b, d));
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));  // rho is a caller buffer
    return MG_OK;
}

int mg_batch_set_design_device(mg_batch *b, int32_t d, const double *rho_dev) {
    if (!b || !rho_dev || d < 0 || d >= b->n_designs) return MG_EINVAL;
    const int64_t ne = (int64_t)b->nx[d] * b->ny[d] * b->nz[d];
    MG_CUDA_TRY(cudaMemsetAsync(b->d_status, 0, sizeof(int), b->stream));
    MG_CUDA_TRY(cudaMemcpyAsync(b->d_rho + b->rho_off[d], rho_dev, ne * 8, cudaMemcpyDeviceToDevice, b->stream));
    MG_TRY(refresh_moduli(b, d));
    return read_device_status(b);
}

int mg_batch_solve(mg_batch *b, const mg_solve_opts *opts, mg_solve_report *reports) {
    if (!b || !opts) return MG_EINVAL;
    return batch_solve(b, *opts, nullptr, reports);
}

int mg_batch_solve_subset(mg_batch *b, const mg_solve_opts *opts, const uint8_t *active,
                          mg_solve_report *reports) {
    if (!b || !opts || !active) return MG_EINVAL;
    return batch_solve(b, *opts, active, reports);
}

int mg_batch_results(mg_batch *b, int32_t d, double *compliance, double *dc, double *u) {
    if (!b || d < 0 || d >= b->n_designs) return MG_EINVAL;
    const int64_t ne = (int64_t)b->nx[d] * b->ny[d] * b->nz[d];
    const int64_t nd = dofs_of(b->nx[d], b->ny[d], b->nz[d]);
    for (int c = 0; c < b->cases[d]; c++) {
        const int i = b->first[d] + c;
        if (compliance) compliance[c] = b->compliance[i];
        if (dc)
            MG_CUDA_TRY(cudaMemcpyAsync(dc + c * ne, b->d_dc + b->dc_off[i], ne * 8, cudaMemcpyDeviceToHost,
                                        b->stream));
        if (u) {
            MG_TRY(mf_batch_get_u(b->mf, i, b->d_u));
            MG_CUDA_TRY(cudaMemcpyAsync(u + c * nd, b->d_u, nd * 8, cudaMemcpyDeviceToHost, b->stream));
            MG_CUDA_TRY(cudaStreamSynchronize(b->stream));  // d_u is reused per case
        }
    }
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return MG_OK;
}

int mg_batch_autotune(mg_batch *b, mg_solve_opts *opts, int32_t max_trials, double *seconds) {
    if (!b || !opts) return MG_EINVAL;
    if (opts->precision < MG_MIXED_TF32 || opts->precision > MG_MIXED_BF16X3) {
        set_error("the autotuner tunes the mixed-precision forms");
        return MG_ENOTSUP;
    }
    const std::string key = tune_key(b, *opts);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        tune_file_load();
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            apply_entry(it->second, *opts);
            if (seconds) *seconds = it->second.seconds;
            return MG_OK;
        }
    }
    // trial set: the first case of the first design of every distinct shape
    std::vector<uint8_t> active(b->n_probs, 0);
    {
        std::vector<std::string> seen;
        for (int d = 0; d < b->n_designs; d++) {
            char s[64];
            snprintf(s, sizeof(s), "%dx%dx%d", b->nx[d], b->ny[d], b->nz[d]);
            if (std::find(seen.begin(), seen.end(), s) != seen.end()) continue;
            seen.push_back(s);
            active[b->first[d]] = 1;
        }
    }
    const bool bf16 = (opts->precision == MG_MIXED_BF16 || opts->precision == MG_MIXED_BF16X3);
    TuneEntry cur{opts->precision, opts->smooth_degree > 0 ? opts->smooth_degree : 2,
                  opts->coarse_degree > 0 ? opts->coarse_degree : 8,
                  opts->graph_chunk > 0 ? opts->graph_chunk : 2,
                  opts->vec_blocks_per_sm > 0 ? opts->vec_blocks_per_sm : 8,
                  opts->inner_rtol > 0 ? opts->inner_rtol : 1e-3, 0.0,
                  opts->smoother_operator == MG_SMOOTHER_TENSOR ? MG_SMOOTHER_TENSOR : MG_SMOOTHER_FACTORED};
    int trials = 0;
    const int cap = max_trials > 0 ? max_trials : 16;
    auto run = [&](const TuneEntry &e) -> double {
        mg_solve_opts o = *opts;
        apply_entry(e, o);
        o.warm_start = 0;
        double best = 1e30;
        for (int r = 0; r < 2; r++) {  // best of two: the first run also captures the graph
            const double t0 = wall_time();
            const int rc = batch_solve(b, o, active.data(), nullptr);
            const double t = wall_time() - t0;
            if (rc != MG_OK) return 1e30;
            best = std::min(best, t);
        }
        trials++;
        return best;
    };
    cur.seconds = run(cur);
    if (cur.seconds >= 1e30) {
        set_error("autotuner: the starting schedule does not converge");
        return MG_ENOCONV;
    }
    // coordinate search over one knob at a time, keeping improvements
    const int precs[2] = {bf16 ? MG_MIXED_BF16X3 : MG_MIXED_TF32X3, bf16 ? MG_MIXED_BF16 : MG_MIXED_TF32};
    const int smooths[3] = {1, 2, 3};
    const int coarses[3] = {4, 8, 16};
    const int chunks[3] = {2, 4, 8};
    const int vecs[3] = {4, 8, 16};
    const double inners[3] = {1e-2, 1e-3, 1e-4};
    const int smoothers[2] = {MG_SMOOTHER_FACTORED, MG_SMOOTHER_TENSOR};
    for (int knob = 0; knob < 7 && trials < cap; knob++) {
        const int nvals = (knob == 0 || knob == 6) ? 2 : 3;
        for (int v = 0; v < nvals && trials < cap; v++) {
            TuneEntry t = cur;
            switch (knob) {
                case 0: t.precision = precs[v]; break;
                case 1: t.smooth = smooths[v]; break;
                case 2: t.coarse = coarses[v]; break;
                case 3: t.chunk = chunks[v]; break;
                case 4: t.vec_blocks = vecs[v]; break;
                case 5: t.inner_rtol = inners[v]; break;
                default: t.smoother = smoothers[v]; break;
            }
            if (t.precision == cur.precision && t.smooth == cur.smooth && t.coarse == cur.coarse &&
                t.chunk == cur.chunk && t.vec_blocks == cur.vec_blocks && t.inner_rtol == cur.inner_rtol &&
                t.smoother == cur.smoother)
                continue;
            t.seconds = run(t);
            if (t.seconds < cur.seconds) cur = t;
        }
    }
    // trials leave the batch's solutions and results stale
    for (int i = 0; i < b->n_probs; i++)
        if (active[i]) b->reports[i] = mg_solve_report{};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = cur;
        tune_file_save();
    }
    apply_entry(cur, *opts);
    if (seconds) *seconds = cur.seconds;
    return MG_OK;
}

}  // extern "C"
