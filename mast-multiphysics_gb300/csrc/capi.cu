// capi.cu -- host side of the C ABI (include/mastgpu.h): problem set-up
// (sparsity pattern, colouring, Dirichlet elimination tables, element->CSR
// maps), the Newton/Krylov drivers and the output/sensitivity entry points.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "mg_internal.h"

namespace mg {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
static std::atomic<int> g_alloc_countdown{-1};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

double wall_time() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

int dev_alloc(void **ptr, size_t bytes) {
    *ptr = nullptr;
    int c = g_alloc_countdown.load();
    if (c >= 0) {
        if (c == 0) {
            set_error("injected allocation failure (%zu bytes)", bytes);
            return MG_ENOMEM;
        }
        g_alloc_countdown.store(c - 1);
    }
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? MG_ENOMEM : MG_ECUDA;
    }
    return MG_OK;
}

void dev_free(void *ptr) {
    if (ptr) cudaFree(ptr);
}

namespace {

__global__ void axpy_kernel(int64_t n, double a, const double *__restrict__ x,
                            double *__restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fma(a, x[i], y[i]);
}

__global__ void masked_neg_kernel(int64_t n, const double *__restrict__ x,
                                  const uint8_t *__restrict__ fixed, double *__restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (fixed && fixed[i]) ? 0.0 : -x[i];
}

inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <class F>
void parallel_for(int64_t n, F f) {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 4096 || nt == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back(f, b, e);
    }
    for (auto &t : th) t.join();
}

// node adjacency through shared elements (sorted, unique, includes self)
void node_adjacency(int npe, int64_t n_nodes, int64_t n_elems, const int32_t *conn,
                    std::vector<int64_t> &aptr, std::vector<int32_t> &adj) {
    std::vector<int64_t> eptr(n_nodes + 1, 0);
    for (int64_t e = 0; e < n_elems; e++)
        for (int a = 0; a < npe; a++) eptr[conn[e * npe + a] + 1]++;
    for (int64_t i = 0; i < n_nodes; i++) eptr[i + 1] += eptr[i];
    std::vector<int32_t> elist(eptr[n_nodes]);
    {
        std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
        for (int64_t e = 0; e < n_elems; e++)
            for (int a = 0; a < npe; a++) elist[fill[conn[e * npe + a]]++] = (int32_t)e;
    }
    std::vector<int32_t> deg(n_nodes);
    std::vector<std::vector<int32_t>> tmp(n_nodes);
    parallel_for(n_nodes, [&](int64_t b, int64_t e) {
        std::vector<int32_t> buf;
        for (int64_t n = b; n < e; n++) {
            buf.clear();
            for (int64_t k = eptr[n]; k < eptr[n + 1]; k++) {
                const int32_t *en = conn + (int64_t)elist[k] * npe;
                buf.insert(buf.end(), en, en + npe);
            }
            std::sort(buf.begin(), buf.end());
            buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
            tmp[n] = buf;
            deg[n] = (int32_t)buf.size();
        }
    });
    aptr.assign(n_nodes + 1, 0);
    for (int64_t n = 0; n < n_nodes; n++) aptr[n + 1] = aptr[n] + deg[n];
    adj.resize(aptr[n_nodes]);
    parallel_for(n_nodes, [&](int64_t b, int64_t e) {
        for (int64_t n = b; n < e; n++) std::copy(tmp[n].begin(), tmp[n].end(), adj.begin() + aptr[n]);
    });
}

int upload(void **dst, const void *src, size_t bytes, cudaStream_t s) {
    MG_TRY(dev_alloc(dst, bytes));
    if (bytes) MG_CUDA_TRY(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s));
    return MG_OK;
}

int release(mg_problem *p) {
    if (!p) return MG_OK;
    if (p->stream) cudaStreamSynchronize(p->stream);
    krylov_free(p);
    matfree_free(p);
    void *ptrs[] = {p->d_coords, p->d_conn, p->d_color_elems, p->d_fixed, p->d_F, p->d_rho,
                    p->d_E, p->d_dE, p->d_s, p->d_q, p->d_conv_mask, p->A.rowptr, p->A.cols,
                    p->A.vals, p->d_emap, p->d_fix_zero, p->d_fix_diag, p->d_X, p->d_R,
                    p->d_tmp, p->d_tmp2, p->d_elem_out, p->d_red, p->d_ks, p->d_side, p->d_rho_nodes,
                    p->d_Eq, p->d_dEq, p->d_qp_out, p->d_node_out, p->d_node_inc_ptr, p->d_node_inc};
    for (void *q : ptrs) dev_free(q);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return MG_OK;
}

int to_device_vec(mg_problem *p, const double *host, double *dev, int64_t n) {
    MG_CUDA_TRY(cudaMemcpyAsync(dev, host, n * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    return MG_OK;
}

int to_host_vec(mg_problem *p, const double *dev, double *host, int64_t n) {
    MG_CUDA_TRY(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

bool finite_all(const double *v, int64_t n) {
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(v[i])) return false;
    return true;
}

int create_impl(const mg_mesh_desc *mesh, const mg_material_desc *mat, const mg_bc_desc *bc,
                mg_problem *p) {
    p->physics = mesh->physics;
    switch (mesh->physics) {
        case MG_PHYSICS_ELASTICITY_HEX8:
        case MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR: p->dim = 3; p->npe = 8; p->dpn = 3; break;
        case MG_PHYSICS_MEMBRANE_QUAD4: p->dim = 2; p->npe = 4; p->dpn = 2; break;
        case MG_PHYSICS_HEAT_QUAD4: p->dim = 2; p->npe = 4; p->dpn = 1; break;
        default: set_error("unknown physics %d", mesh->physics); return MG_EINVAL;
    }
    const int64_t nn = mesh->n_nodes, ne = mesh->n_elems;
    if (nn <= 0 || ne <= 0 || !mesh->coords || !mesh->conn) {
        set_error("empty mesh");
        return MG_EINVAL;
    }
    if (nn * p->dpn >= INT32_MAX) {
        set_error("mesh too large for int32 CSR indices");
        return MG_EINVAL;
    }
    p->n_nodes = nn;
    p->n_elems = ne;
    p->n_dofs = nn * p->dpn;
    p->grid_nx = mesh->grid_nx;
    p->grid_ny = mesh->grid_ny;
    p->grid_nz = mesh->grid_nz;
    p->mat = *mat;
    if (!(mat->E0 > 0) && p->physics != MG_PHYSICS_HEAT_QUAD4) {
        set_error("E0 must be positive");
        return MG_EINVAL;
    }
    if (p->dim == 2 && !(mat->thickness > 0)) {
        set_error("2D section thickness must be positive");
        return MG_EINVAL;
    }
    p->h_coords.assign(mesh->coords, mesh->coords + nn * p->dim);
    p->h_conn.assign(mesh->conn, mesh->conn + ne * p->npe);
    if (!finite_all(p->h_coords.data(), nn * p->dim)) {
        set_error("non-finite node coordinates");
        return MG_EINVAL;
    }
    for (int32_t c : p->h_conn)
        if (c < 0 || c >= nn) {
            set_error("connectivity entry %d outside [0, %lld)", c, (long long)nn);
            return MG_EINVAL;
        }
    MG_CUDA_TRY(cudaGetDevice(&p->device));
    MG_CUDA_TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    cudaStream_t s = p->stream;

    // ---- boundary conditions ----
    p->h_fixed.assign(p->n_dofs, 0);
    p->h_F.assign(p->n_dofs, 0.0);
    std::vector<uint8_t> conv_mask;
    if (bc) {
        for (int64_t i = 0; i < bc->n_fixed; i++) {
            int64_t d = bc->fixed_dofs[i];
            if (d < 0 || d >= p->n_dofs) { set_error("fixed dof %lld out of range", (long long)d); return MG_EINVAL; }
            p->h_fixed[d] = 1;
        }
        for (int64_t i = 0; i < bc->n_point_loads; i++) {
            int64_t d = bc->load_dofs[i];
            if (d < 0 || d >= p->n_dofs || !std::isfinite(bc->load_values[i])) {
                set_error("bad point load %lld", (long long)i);
                return MG_EINVAL;
            }
            p->h_F[d] += bc->load_values[i];
        }
        if (bc->n_conv > 0) {
            if (p->physics != MG_PHYSICS_HEAT_QUAD4) { set_error("convection needs heat physics"); return MG_EINVAL; }
            conv_mask.assign(ne, 0);
            for (int64_t i = 0; i < bc->n_conv; i++) {
                int32_t e = bc->conv_elems[i], sd = bc->conv_sides[i];
                if (e < 0 || e >= ne || sd < 0 || sd > 3) { set_error("bad convection side %lld", (long long)i); return MG_EINVAL; }
                conv_mask[e] |= (uint8_t)(1u << sd);
            }
            p->conv_h = bc->conv_h;
            p->conv_Tinf = bc->conv_Tinf;
            p->n_conv = bc->n_conv;
        }
        if (bc->source_elem) {
            if (!finite_all(bc->source_elem, ne)) { set_error("non-finite heat source"); return MG_EINVAL; }
            MG_TRY(upload(reinterpret_cast<void **>(&p->d_q), bc->source_elem, ne * sizeof(double), s));
        }
    }
    for (int64_t d = 0; d < p->n_dofs; d++)
        if (p->h_fixed[d]) p->h_F[d] = 0.0;
    p->h_F_point = p->h_F;

    // ---- colouring (no two elements of a colour share a node) ----
    std::vector<int32_t> color(ne, 0);
    const bool structured = p->grid_nx > 0 && p->grid_ny > 0 &&
                            (p->dim == 2 ? (int64_t)p->grid_nx * p->grid_ny == ne
                                         : p->grid_nz > 0 &&
                                               (int64_t)p->grid_nx * p->grid_ny * p->grid_nz == ne);
    if (structured) {
        for (int64_t e = 0; e < ne; e++) {
            int64_t i = e % p->grid_nx, j = (e / p->grid_nx) % p->grid_ny;
            int64_t k = p->dim == 3 ? e / ((int64_t)p->grid_nx * p->grid_ny) : 0;
            color[e] = (int32_t)((i & 1) | (j & 1) << 1 | (k & 1) << 2);
        }
        p->n_colors = p->dim == 3 ? 8 : 4;
    } else {
        std::vector<uint64_t> used(nn, 0);
        int ncol = 0;
        for (int64_t e = 0; e < ne; e++) {
            uint64_t m = 0;
            for (int a = 0; a < p->npe; a++) m |= used[p->h_conn[e * p->npe + a]];
            int c = 0;
            while (c < 64 && (m >> c & 1ull)) c++;
            if (c == 64) { set_error("element colouring needs more than 64 colours"); return MG_ENOTSUP; }
            color[e] = c;
            ncol = std::max(ncol, c + 1);
            for (int a = 0; a < p->npe; a++) used[p->h_conn[e * p->npe + a]] |= 1ull << c;
        }
        p->n_colors = ncol;
    }
    // verify the structured colouring (it relies on the libMesh grid numbering)
    if (structured) {
        std::vector<int64_t> stamp(nn, -1);
        for (int c = 0; c < p->n_colors; c++)
            for (int64_t e = 0; e < ne; e++) {
                if (color[e] != c) continue;
                for (int a = 0; a < p->npe; a++) {
                    int32_t nd = p->h_conn[e * p->npe + a];
                    if (stamp[nd] == c) { set_error("grid dims do not match the connectivity"); return MG_EINVAL; }
                    stamp[nd] = c;
                }
            }
    }
    p->color_ptr.assign(p->n_colors + 1, 0);
    for (int64_t e = 0; e < ne; e++) p->color_ptr[color[e] + 1]++;
    for (int c = 0; c < p->n_colors; c++) p->color_ptr[c + 1] += p->color_ptr[c];
    std::vector<int32_t> celems(ne);
    {
        std::vector<int64_t> fill(p->color_ptr.begin(), p->color_ptr.end() - 1);
        for (int64_t e = 0; e < ne; e++) celems[fill[color[e]]++] = (int32_t)e;
    }

    // ---- sparsity pattern (node-interleaved, shared column list per node) ----
    std::vector<int64_t> aptr;
    std::vector<int32_t> adj;
    node_adjacency(p->npe, nn, ne, p->h_conn.data(), aptr, adj);
    const int dpn = p->dpn;
    const int64_t n = p->n_dofs;
    std::vector<int32_t> rowptr(n + 1);
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int64_t nd = 0; nd < nn; nd++) {
        int64_t deg = aptr[nd + 1] - aptr[nd];
        for (int c = 0; c < dpn; c++) {
            nnz += deg * dpn;
            if (nnz >= INT32_MAX) { set_error("nnz exceeds int32 range"); return MG_ENOTSUP; }
            rowptr[nd * dpn + c + 1] = (int32_t)nnz;
        }
    }
    std::vector<int32_t> cols(nnz);
    parallel_for(nn, [&](int64_t b, int64_t e) {
        for (int64_t nd = b; nd < e; nd++) {
            int64_t deg = aptr[nd + 1] - aptr[nd];
            for (int c = 0; c < dpn; c++) {
                int32_t *dst = cols.data() + rowptr[nd * dpn + c];
                for (int64_t k = 0; k < deg; k++)
                    for (int d = 0; d < dpn; d++) dst[k * dpn + d] = adj[aptr[nd] + k] * dpn + d;
            }
        }
    });
    p->A.n = n;
    p->A.nnz = nnz;
    p->A.dpn = dpn;

    // ---- Dirichlet elimination tables ----
    std::vector<int64_t> fix_zero, fix_diag;
    for (int64_t nd = 0; nd < nn; nd++) {
        for (int c = 0; c < dpn; c++) {
            int64_t row = nd * dpn + c;
            if (p->h_fixed[row]) {
                for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++)
                    (cols[k] == row ? fix_diag : fix_zero).push_back(k);
            }
        }
    }
    for (int64_t nd = 0; nd < nn; nd++) {
        bool any = false;
        for (int c = 0; c < dpn; c++) any |= p->h_fixed[nd * dpn + c] != 0;
        if (!any) continue;
        for (int64_t k = aptr[nd]; k < aptr[nd + 1]; k++) {
            int32_t m = adj[k];
            // position of node nd in m's adjacency
            auto it = std::lower_bound(adj.begin() + aptr[m], adj.begin() + aptr[m + 1], (int32_t)nd);
            int64_t idx = it - (adj.begin() + aptr[m]);
            for (int i = 0; i < dpn; i++) {
                int64_t row = (int64_t)m * dpn + i;
                if (p->h_fixed[row]) continue;
                for (int c = 0; c < dpn; c++)
                    if (p->h_fixed[nd * dpn + c]) fix_zero.push_back(rowptr[row] + idx * dpn + c);
            }
        }
    }
    p->n_fix_zero = (int64_t)fix_zero.size();
    p->n_fix_diag = (int64_t)fix_diag.size();

    // ---- uploads ----
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_coords), p->h_coords.data(), p->h_coords.size() * 8, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_conn), p->h_conn.data(), p->h_conn.size() * 4, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_color_elems), celems.data(), celems.size() * 4, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_fixed), p->h_fixed.data(), p->h_fixed.size(), s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_F), p->h_F.data(), p->h_F.size() * 8, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->A.rowptr), rowptr.data(), rowptr.size() * 4, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->A.cols), cols.data(), cols.size() * 4, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_fix_zero), fix_zero.data(), fix_zero.size() * 8, s));
    MG_TRY(upload(reinterpret_cast<void **>(&p->d_fix_diag), fix_diag.data(), fix_diag.size() * 8, s));
    if (!conv_mask.empty())
        MG_TRY(upload(reinterpret_cast<void **>(&p->d_conv_mask), conv_mask.data(), conv_mask.size(), s));
    MG_TRY(dev_alloc_n(&p->A.vals, (size_t)nnz));
    MG_TRY(dev_alloc_n(&p->d_emap, (size_t)ne * p->npe * p->npe));
    MG_TRY(dev_alloc_n(&p->d_rho, (size_t)ne));
    MG_TRY(dev_alloc_n(&p->d_E, (size_t)ne));
    MG_TRY(dev_alloc_n(&p->d_dE, (size_t)ne));
    MG_TRY(dev_alloc_n(&p->d_elem_out, (size_t)ne));
    MG_TRY(dev_alloc_n(&p->d_X, (size_t)n));
    MG_TRY(dev_alloc_n(&p->d_R, (size_t)n));
    MG_TRY(dev_alloc_n(&p->d_tmp, (size_t)n));
    MG_TRY(dev_alloc_n(&p->d_tmp2, (size_t)std::max<int64_t>(n, ne) + 1024));
    p->red_blocks = 152 * 8;
    MG_TRY(dev_alloc_n(&p->d_red, (size_t)2 * p->red_blocks + 16));
    MG_CUDA_TRY(cudaMemsetAsync(p->d_X, 0, n * 8, s));
    {
        std::vector<double> ones(ne, 1.0);
        MG_CUDA_TRY(cudaMemcpyAsync(p->d_rho, ones.data(), ne * 8, cudaMemcpyHostToDevice, s));
        if (p->physics == MG_PHYSICS_HEAT_QUAD4) {
            MG_TRY(dev_alloc_n(&p->d_s, (size_t)ne));
            MG_CUDA_TRY(cudaMemcpyAsync(p->d_s, ones.data(), ne * 8, cudaMemcpyHostToDevice, s));
        }
        if (p->physics != MG_PHYSICS_HEAT_QUAD4) MG_TRY(compute_modulus(p));
        MG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    MG_TRY(build_emap(p));
    MG_TRY(krylov_init(p));
    MG_CUDA_TRY(cudaStreamSynchronize(s));
    return MG_OK;
}

int newton_solve(mg_problem *p, const mg_solve_opts &o, mg_solve_report *rep) {
    // NonlinearSystem::solve under SNES Newton: J dX = -R, X += dX (heat conduction and the
    // nonlinear-strain HEX8 element)
    double r0 = -1.0, rn = 0.0;
    int kry = 0, it_newton = 0, rc = MG_OK;
    const int maxn = o.max_newton > 0 ? o.max_newton : 30;
    for (it_newton = 0;; it_newton++) {
        MG_TRY(assemble_system(p, p->d_X, p->d_R, true, o.consistent_jacobian != 0));
        MG_TRY(dot(p, p->d_R, p->d_R, p->n_dofs, &rn));
        rn = sqrt(rn);
        if (r0 < 0) r0 = rn;
        if (rn <= o.newton_rtol * r0 || rn == 0.0 || it_newton >= maxn) break;
        MG_CUDA_TRY(cudaMemsetAsync(p->d_tmp, 0, p->n_dofs * 8, p->stream));
        int its = 0;
        double rr = 0;
        rc = krylov_solve(p, p->A, p->d_R, p->d_tmp, o, o.krylov, &its, &rr);
        kry += its;
        if (rc != MG_OK) break;
        axpy_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(p->n_dofs, -1.0, p->d_tmp, p->d_X);
        MG_CUDA_TRY(cudaGetLastError());
    }
    if (rep) {
        rep->newton_iterations = it_newton;
        rep->krylov_iterations = kry;
        rep->residual_norm = rn;
        rep->relres = r0 > 0 ? rn / r0 : 0.0;
    }
    if (rc == MG_OK && it_newton >= maxn && rn > o.newton_rtol * r0) rc = MG_ENOCONV;
    return rc;
}

int solve_linear(mg_problem *p, const mg_solve_opts &o, mg_solve_report *rep) {
    if (!p->jacobian_valid) count_launches(p->n_colors + 2);
    MG_TRY(assemble_system(p, p->d_X, nullptr, true, false));
    int its = 0;
    double rr = 0;
    int rc = krylov_solve(p, p->A, p->d_F, p->d_X, o, o.krylov, &its, &rr);
    // true FP64 residual ||F - K u|| / ||F||
    MG_TRY(spmv(p, p->A, p->d_X, p->d_tmp));
    axpy_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(p->n_dofs, -1.0, p->d_F, p->d_tmp);
    MG_CUDA_TRY(cudaGetLastError());
    double rn2 = 0, fn2 = 0;
    MG_TRY(dot(p, p->d_tmp, p->d_tmp, p->n_dofs, &rn2));
    MG_TRY(dot(p, p->d_F, p->d_F, p->n_dofs, &fn2));
    if (rep) {
        rep->newton_iterations = 1;
        rep->krylov_iterations = its;
        rep->residual_norm = sqrt(rn2);
        rep->relres = fn2 > 0 ? sqrt(rn2 / fn2) : sqrt(rn2);
    }
    return rc;
}

}  // namespace
}  // namespace mg

using namespace mg;

extern "C" {

namespace {
// entry points whose element kernels take one modulus per element
int element_design_only(mg_problem *p, const char *what) {
    if (p && p->nodal_design) {
        set_error("%s: takes element densities (the problem has a nodal density field)", what);
        return MG_ENOTSUP;
    }
    return MG_OK;
}
}  // namespace

int mg_version(void) { return MG_ABI_VERSION; }

const char *mg_status_string(int s) {
    switch (s) {
        case MG_OK: return "ok";
        case MG_EINVAL: return "invalid argument";
        case MG_ENOMEM: return "out of device memory";
        case MG_ENOCONV: return "not converged";
        case MG_EBREAKDOWN: return "Krylov breakdown";
        case MG_ENAN: return "NaN/Inf in reduction";
        case MG_ETIMEDOUT: return "timed out";
        case MG_ECUDA: return "CUDA error";
        case MG_ENOTSUP: return "not supported";
        case MG_EBUSY: return "busy";
        case MG_EBADELEM: return "degenerate element";
        default: return "unknown status";
    }
}

const char *mg_last_error(void) { return g_err; }

// Host-side fault injection for tests: the countdown-th next device allocation
// made by this library fails with MG_ENOMEM (-1 disables).
void mg_debug_fail_alloc_after(int countdown) { g_alloc_countdown.store(countdown); }

int mg_device_info(char *name, int name_len, int *sm_count, int *cc_major, int *cc_minor) {
    int dev = 0;
    cudaDeviceProp prop;
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    if (name && name_len > 0) snprintf(name, name_len, "%s", prop.name);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    return MG_OK;
}

void mg_default_solve_opts(mg_solve_opts *o) {
    memset(o, 0, sizeof(*o));
    o->precision = MG_PLAIN_FP64;
    o->krylov = MG_KRYLOV_CG;
    o->max_iterations = 200000;
    o->max_newton = 30;
    o->rtol = 1e-10;
    o->newton_rtol = 1e-10;
    o->consistent_jacobian = 1;
    o->max_refinements = 30;
    o->inner_rtol = 1e-4;
    o->timeout_s = 0.0;
    o->warm_start = 0;
    o->graph_chunk = 0;
    o->preconditioner = MG_PC_MULTIGRID;
    o->smooth_degree = 2;
    o->coarse_degree = 8;
}

int mg_problem_create(const mg_mesh_desc *mesh, const mg_material_desc *mat, const mg_bc_desc *bc,
                      mg_problem **out) {
    if (!mesh || !mat || !out) {
        set_error("null argument");
        return MG_EINVAL;
    }
    *out = nullptr;
    mg_problem *p = new mg_problem();
    int rc = create_impl(mesh, mat, bc, p);
    if (rc != MG_OK) {
        char saved[512];
        snprintf(saved, sizeof(saved), "%s", g_err);
        release(p);
        snprintf(g_err, sizeof(g_err), "%s", saved);
        return rc;
    }
    *out = p;
    return MG_OK;
}

void mg_problem_destroy(mg_problem *p) { release(p); }

int mg_problem_info(const mg_problem *p, int64_t *n_dofs, int64_t *nnz, int32_t *n_colors) {
    if (!p) return MG_EINVAL;
    if (n_dofs) *n_dofs = p->n_dofs;
    if (nnz) *nnz = p->A.nnz;
    if (n_colors) *n_colors = p->n_colors;
    return MG_OK;
}

void *mg_problem_stream(mg_problem *p) { return p ? (void *)p->stream : nullptr; }

int mg_set_design(mg_problem *p, const double *rho) {
    if (!p || !rho) return MG_EINVAL;
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) { set_error("heat physics has no density design"); return MG_ENOTSUP; }
    MG_TRY(to_device_vec(p, rho, p->d_rho, p->n_elems));
    // the modulus kernel flags densities outside [0,1] (or NaN); the host looks for
    // the first one only then, for the message
    const int rc = compute_modulus(p);
    if (rc == MG_EINVAL)
        for (int64_t e = 0; e < p->n_elems; e++)
            if (!(rho[e] >= 0.0 && rho[e] <= 1.0)) {
                set_error("density %lld = %g outside [0,1]", (long long)e, rho[e]);
                break;
            }
    MG_TRY(rc);
    p->nodal_design = false;
    p->jacobian_valid = false;
    return MG_OK;
}

int mg_set_design_device(mg_problem *p, const double *rho_dev) {
    if (!p || !rho_dev) return MG_EINVAL;
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) return MG_ENOTSUP;
    MG_CUDA_TRY(cudaMemcpyAsync(p->d_rho, rho_dev, p->n_elems * 8, cudaMemcpyDeviceToDevice, p->stream));
    MG_TRY(compute_modulus(p));
    p->nodal_design = false;
    p->jacobian_valid = false;
    return MG_OK;
}

int mg_set_design_nodal(mg_problem *p, const double *rho_nodes) {
    // the MeshFieldFunction density of example_6.cpp:104-137 (FIRST-order LAGRANGE
    // "rho", :250-252): the modulus at each Gauss point from the trilinear field there
    if (!p || !rho_nodes) {
        set_error("mg_set_design_nodal: invalid argument");
        return MG_EINVAL;
    }
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8) {
        set_error("a nodal density field needs the linear-strain HEX8 physics");
        return MG_ENOTSUP;
    }
    for (int64_t n = 0; n < p->n_nodes; n++)
        if (!(rho_nodes[n] >= 0.0 && rho_nodes[n] <= 1.0)) {
            set_error("nodal density %lld = %g outside [0,1]", (long long)n, rho_nodes[n]);
            return MG_EINVAL;
        }
    if (!p->d_node_inc) {  // the last buffer allocated: a failed first call is retried whole
        if (!p->d_rho_nodes) MG_TRY(dev_alloc_n(&p->d_rho_nodes, (size_t)p->n_nodes));
        if (!p->d_node_out) MG_TRY(dev_alloc_n(&p->d_node_out, (size_t)p->n_nodes));
        if (!p->d_Eq) MG_TRY(dev_alloc_n(&p->d_Eq, (size_t)p->n_elems * 8));
        if (!p->d_dEq) MG_TRY(dev_alloc_n(&p->d_dEq, (size_t)p->n_elems * 8));
        if (!p->d_qp_out) MG_TRY(dev_alloc_n(&p->d_qp_out, (size_t)p->n_elems * 8));
        // node -> (element, corner) incidences in element order
        std::vector<int32_t> ptr(p->n_nodes + 1, 0), inc((size_t)p->n_elems * 8);
        for (int64_t k = 0; k < p->n_elems * 8; k++) ptr[p->h_conn[k] + 1]++;
        for (int64_t n = 0; n < p->n_nodes; n++) ptr[n + 1] += ptr[n];
        std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
        for (int64_t k = 0; k < p->n_elems * 8; k++) inc[fill[p->h_conn[k]]++] = (int32_t)k;
        if (!p->d_node_inc_ptr) MG_TRY(dev_alloc_n(&p->d_node_inc_ptr, ptr.size()));
        int32_t *inc_dev = nullptr;
        MG_TRY(dev_alloc_n(&inc_dev, inc.size()));
        cudaError_t e = cudaMemcpyAsync(p->d_node_inc_ptr, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice,
                                        p->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(inc_dev, inc.data(), inc.size() * 4, cudaMemcpyHostToDevice, p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);  // ptr / inc are host temporaries
        if (e != cudaSuccess) {
            dev_free(inc_dev);
            set_error("nodal design tables: %s", cudaGetErrorString(e));
            return MG_ECUDA;
        }
        p->d_node_inc = inc_dev;
    }
    MG_TRY(to_device_vec(p, rho_nodes, p->d_rho_nodes, p->n_nodes));
    MG_TRY(compute_nodal_modulus(p));
    p->nodal_design = true;
    p->jacobian_valid = false;
    return MG_OK;
}

int mg_set_elem_scale(mg_problem *p, const double *s) {
    if (!p || !s) return MG_EINVAL;
    if (p->physics != MG_PHYSICS_HEAT_QUAD4) return MG_ENOTSUP;
    if (!finite_all(s, p->n_elems)) { set_error("non-finite element scale"); return MG_EINVAL; }
    MG_TRY(to_device_vec(p, s, p->d_s, p->n_elems));
    p->jacobian_valid = false;
    return MG_OK;
}

int mg_residual_and_jacobian(mg_problem *p, const double *X, double *R, int assemble_jacobian) {
    if (!p || !X) return MG_EINVAL;
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) p->jacobian_valid = false;
    MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
    MG_TRY(assemble_system(p, p->d_tmp, R ? p->d_R : nullptr, assemble_jacobian != 0, true));
    if (R) MG_TRY(to_host_vec(p, p->d_R, R, p->n_dofs));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int mg_get_csr(mg_problem *p, int32_t *rowptr, int32_t *cols, double *vals) {
    if (!p) return MG_EINVAL;
    if (rowptr)
        MG_CUDA_TRY(cudaMemcpyAsync(rowptr, p->A.rowptr, (p->A.n + 1) * 4, cudaMemcpyDeviceToHost, p->stream));
    if (cols)
        MG_CUDA_TRY(cudaMemcpyAsync(cols, p->A.cols, p->A.nnz * 4, cudaMemcpyDeviceToHost, p->stream));
    if (vals)
        MG_CUDA_TRY(cudaMemcpyAsync(vals, p->A.vals, p->A.nnz * 8, cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int mg_element_matrices(mg_problem *p, const double *X, int64_t first, int64_t count, double *Ke,
                        double *fe) {
    if (!p || first < 0 || count <= 0 || first + count > p->n_elems || !Ke) return MG_EINVAL;
    const int nd = p->npe * p->dpn;
    double *dK = nullptr, *df = nullptr;
    MG_TRY(dev_alloc_n(&dK, (size_t)count * nd * nd));
    int rc = dev_alloc_n(&df, (size_t)count * nd);
    if (rc == MG_OK) {
        if (X) rc = to_device_vec(p, X, p->d_tmp, p->n_dofs);
        else if (cudaMemsetAsync(p->d_tmp, 0, p->n_dofs * 8, p->stream) != cudaSuccess) rc = MG_ECUDA;
    }
    if (rc == MG_OK) rc = element_matrices(p, p->d_tmp, first, count, dK, df);
    if (rc == MG_OK) {
        if (cudaMemcpyAsync(Ke, dK, count * nd * nd * 8, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
            (fe && cudaMemcpyAsync(fe, df, count * nd * 8, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess) ||
            cudaStreamSynchronize(p->stream) != cudaSuccess)
            rc = MG_ECUDA;
    }
    cudaStreamSynchronize(p->stream);
    dev_free(dK);
    dev_free(df);
    return rc;
}

int mg_spmv(mg_problem *p, const double *x, double *y) {
    if (!p || !x || !y) return MG_EINVAL;
    MG_TRY(to_device_vec(p, x, p->d_tmp, p->n_dofs));
    MG_TRY(spmv(p, p->A, p->d_tmp, p->d_R));
    return to_host_vec(p, p->d_R, y, p->n_dofs);
}

int mg_solve(mg_problem *p, const mg_solve_opts *opts, double *X, mg_solve_report *rep) {
    if (!p) return MG_EINVAL;
    mg_solve_opts o;
    if (opts) o = *opts; else mg_default_solve_opts(&o);
    mg_solve_report r{};
    const double t0 = wall_time();
    if (!o.warm_start) {
        if (X) MG_TRY(to_device_vec(p, X, p->d_X, p->n_dofs));
        else MG_CUDA_TRY(cudaMemsetAsync(p->d_X, 0, p->n_dofs * 8, p->stream));
    }
    int rc;
    if (o.precision == MG_PLAIN_FP64) {
        rc = (p->physics == MG_PHYSICS_HEAT_QUAD4 || p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR)
                 ? newton_solve(p, o, &r)
                 : solve_linear(p, o, &r);
    } else {
        if (p->physics != MG_PHYSICS_ELASTICITY_HEX8) { set_error("mixed precision needs the linear-strain HEX8 SIMP form"); return MG_ENOTSUP; }
        MG_TRY(element_design_only(p, "the mixed-precision solve"));
        rc = matfree_solve(p, o, &r, !o.warm_start && !X);
    }
    p->last_solve_mixed = (o.precision != MG_PLAIN_FP64);
    if (X && (rc == MG_OK || rc == MG_ENOCONV)) {
        int rc2 = to_host_vec(p, p->d_X, X, p->n_dofs);
        if (rc2 != MG_OK) rc = rc2;
    }
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    r.status = rc;
    r.seconds = wall_time() - t0;
    if (rep) *rep = r;
    return rc;
}

int mg_get_solution(mg_problem *p, double *X) {
    if (!p || !X) return MG_EINVAL;
    return to_host_vec(p, p->d_X, X, p->n_dofs);
}

const double *mg_solution_device(mg_problem *p) { return p ? p->d_X : nullptr; }

int mg_sensitivity_assemble(mg_problem *p, const double *X, int32_t kind, int64_t index,
                            double *dRdp) {
    if (!p || !dRdp) return MG_EINVAL;
    MG_TRY(element_design_only(p, "mg_sensitivity_assemble"));
    const double *dX = p->d_X;
    if (X) {
        MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
        dX = p->d_tmp;
    }
    MG_TRY(assemble_param_residual(p, dX, kind, index, p->d_R));
    return to_host_vec(p, p->d_R, dRdp, p->n_dofs);
}

int mg_compliance(mg_problem *p, const double *X, double *compliance, double *dc) {
    if (!p) return MG_EINVAL;
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8 && p->physics != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR)
        return MG_ENOTSUP;
    const double *dX = p->d_X;
    if (X) {
        MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
        dX = p->d_tmp;
    }
    if (compliance) MG_TRY(dot(p, p->d_F, dX, p->n_dofs, compliance));
    if (dc && p->nodal_design) {
        // one value per node: -u^T dK/drho_n u
        MG_TRY(nodal_compliance_sensitivity(p, dX, p->d_node_out));
        return to_host_vec(p, p->d_node_out, dc, p->n_nodes);
    }
    if (dc && p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        // C = F.u with f_int(u, rho) = F: dC/drho_e = -lambda . d f_int / d rho_e, where
        // K_T(u)^T lambda = F (the tangent is symmetric) and d f_int / d rho_e = dE_e f1_e(u)
        // (AssemblyBase::calculate_output_adjoint_sensitivity, assembly_base.cpp:555-590)
        mg_solve_opts o;
        mg_default_solve_opts(&o);
        o.rtol = 1e-13;
        MG_TRY(assemble_system(p, dX, nullptr, true, true));
        double *lam = p->d_R;
        MG_CUDA_TRY(cudaMemsetAsync(lam, 0, p->n_dofs * 8, p->stream));
        int its = 0;
        double rr = 0;
        MG_TRY(krylov_solve(p, p->A, p->d_F, lam, o, MG_KRYLOV_CG, &its, &rr));
        MG_TRY(elem_sensitivity(p, dX, lam, MG_PARAM_DENSITY, p->d_elem_out));
        MG_TRY(to_host_vec(p, p->d_elem_out, dc, p->n_elems));
        for (int64_t e = 0; e < p->n_elems; e++) dc[e] = -dc[e];
        return MG_OK;
    }
    if (dc && p->last_solve_mixed && !X) {
        // structured grid after a mixed solve: shared-K0 FP64 sensitivity kernel
        return matfree_sensitivity(p, dc);
    }
    if (dc) {
        // dC/drho_e = -dE_e u_e^T K1_e u_e (compliance adjoint = -u)
        MG_TRY(elem_sensitivity(p, dX, dX, MG_PARAM_DENSITY, p->d_elem_out));
        MG_TRY(to_host_vec(p, p->d_elem_out, dc, p->n_elems));
        for (int64_t e = 0; e < p->n_elems; e++) dc[e] = -dc[e];
    }
    return MG_OK;
}

int mg_set_side_loads(mg_problem *p, int64_t n, const int32_t *elems, const int32_t *sides,
                      const double *values) {
    // PhysicsDisciplineBase side boundary conditions: "pressure" on HEX8 faces
    // (StructuralElement3D::surface_pressure_residual, solid_element_3d.cpp:815-876) and
    // "heat_flux" on QUAD4 edges (surface_flux_residual, heat_conduction_elem_base.cpp:876-913);
    // replaces the previous side loads, values of a repeated (element, side) add up
    if (!p || n < 0 || (n > 0 && (!elems || !sides || !values))) {
        set_error("mg_set_side_loads: invalid argument");
        return MG_EINVAL;
    }
    int ns;
    if (p->physics == MG_PHYSICS_ELASTICITY_HEX8 || p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) ns = 6;
    else if (p->physics == MG_PHYSICS_HEAT_QUAD4) ns = 4;
    else {
        set_error("side loads: pressure on HEX8 faces or heat flux on QUAD4 edges only");
        return MG_ENOTSUP;
    }
    std::vector<double> h((size_t)p->n_elems * ns, 0.0);
    for (int64_t i = 0; i < n; i++) {
        if (elems[i] < 0 || elems[i] >= p->n_elems || sides[i] < 0 || sides[i] >= ns ||
            !std::isfinite(values[i])) {
            set_error("side load %lld: element %d side %d value %g", (long long)i, elems[i], sides[i], values[i]);
            return MG_EINVAL;
        }
        h[(size_t)elems[i] * ns + sides[i]] += values[i];
    }
    if (!p->d_side) MG_TRY(dev_alloc_n(&p->d_side, h.size()));
    MG_CUDA_TRY(cudaMemcpyAsync(p->d_side, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                p->stream));
    MG_TRY(assemble_side_loads(p));
    matfree_free(p);  // the mixed form copies the load vector when it is set up
    return MG_OK;
}

int mg_ks_stress(mg_problem *p, const double *X, double p_ks, double sigma0, double stress_penalty,
                 double *ks, double *max_vm, double *dks_drho) {
    // KSStressStrainOutput::functional_for_all_elems (ks_stress_output.cpp:41-99) and, for
    // dks_drho, the total derivative of example_6.cpp:798-874: the adjoint term lambda .
    // dR/drho_e (K(X)^T lambda = -dq/dX, the residual at the material's SIMP exponent) plus the
    // direct term through the stress modulus (functional_sensitivity_for_elem, :117-151)
    if (!p || !(p_ks > 0) || !(sigma0 > 0)) return MG_EINVAL;
    MG_TRY(element_design_only(p, "mg_ks_stress"));
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8 && p->physics != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        set_error("the stress output needs HEX8 elasticity");
        return MG_ENOTSUP;
    }
    const double penal = stress_penalty > 0 ? stress_penalty : p->mat.penal;
    if (!p->d_ks) MG_TRY(dev_alloc_n(&p->d_ks, (size_t)6 * p->n_elems + 8));
    const double *dX = p->d_X;
    if (X) {
        MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
        dX = p->d_tmp;
    }
    double red[3] = {0, 0, 0};
    MG_TRY(ks_stress_values(p, dX, p_ks, sigma0, penal, p->d_ks, red));
    const double I = red[0], V = red[1];
    if (!(I > 0) || !std::isfinite(I) || !(V > 0)) {
        set_error("KS sum %g over volume %g (overflow of exp(p (vm - s0)/s0)?)", I, V);
        return MG_ENAN;
    }
    if (ks) *ks = log(I / V) / p_ks;
    if (max_vm) *max_vm = red[2];
    if (!dks_drho) return MG_OK;
    const double inv_s0I = 1.0 / (sigma0 * I);
    // rhs = -dq/dX (zero on constrained dofs) in d_R; lambda in d_tmp2
    MG_TRY(ks_stress_gradient(p, dX, p_ks, sigma0, p->d_ks, inv_s0I, p->d_tmp2));
    masked_neg_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(p->n_dofs, p->d_tmp2, p->d_fixed,
                                                                        p->d_R);
    MG_CUDA_TRY(cudaGetLastError());
    if (p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) p->jacobian_valid = false;
    MG_TRY(assemble_system(p, dX, nullptr, true, true));
    mg_solve_opts o;
    mg_default_solve_opts(&o);
    o.rtol = 1e-13;
    double *lam = p->d_tmp2;
    MG_CUDA_TRY(cudaMemsetAsync(lam, 0, p->n_dofs * 8, p->stream));
    int its = 0;
    double rr = 0;
    MG_TRY(krylov_solve(p, p->A, p->d_R, lam, o, MG_KRYLOV_CG, &its, &rr));
    MG_TRY(elem_sensitivity(p, dX, lam, MG_PARAM_DENSITY, p->d_elem_out));
    MG_TRY(ks_stress_combine(p, p->d_ks, inv_s0I, p->d_elem_out, p->d_elem_out));
    return to_host_vec(p, p->d_elem_out, dks_drho, p->n_elems);
}

int mg_adjoint_solve(mg_problem *p, const double *X, const double *rhs, const mg_solve_opts *opts,
                     double *lambda) {
    // NonlinearSystem::adjoint_solve (nonlinear_system.cpp:798-847): J(X)^T lambda = rhs on the
    // consistent Jacobian; constrained rows give lambda_d = 0
    if (!p || !X || !rhs || !lambda) return MG_EINVAL;
    mg_solve_opts o;
    if (opts) o = *opts; else mg_default_solve_opts(&o);
    std::vector<double> b(rhs, rhs + p->n_dofs);
    for (int64_t i = 0; i < p->n_dofs; i++)
        if (p->h_fixed[i]) b[i] = 0.0;
    MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
    MG_TRY(to_device_vec(p, b.data(), p->d_R, p->n_dofs));
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) p->jacobian_valid = false;
    MG_TRY(assemble_system(p, p->d_tmp, nullptr, true, true));
    double *lam = p->d_tmp2;
    MG_CUDA_TRY(cudaMemsetAsync(lam, 0, p->n_dofs * 8, p->stream));
    int its = 0;
    double rr = 0;
    int rc;
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) {
        CsrMatrix At;
        MG_TRY(transpose_csr(p, p->A, &At));
        rc = krylov_solve(p, At, p->d_R, lam, o, MG_KRYLOV_BICGSTAB, &its, &rr);
        free_csr(&At);
    } else {
        // elasticity: the (tangent) stiffness is symmetric
        rc = krylov_solve(p, p->A, p->d_R, lam, o, o.krylov, &its, &rr);
    }
    if (rc != MG_OK) return rc;
    return to_host_vec(p, lam, lambda, p->n_dofs);
}

int mg_sensitivity_solve(mg_problem *p, const double *X, int32_t kind, int64_t index,
                         const mg_solve_opts *opts, double *du_dp) {
    // NonlinearSystem::sensitivity_solve (nonlinear_system.cpp:741-794): J(X) du/dp = -dR/dp
    // with the Jacobian at X and dR/dp of sensitivity_assemble; constrained rows give 0
    // (enforce_constraints_exactly, homogeneous)
    if (!p || !X || !du_dp) {
        set_error("mg_sensitivity_solve: invalid argument");
        return MG_EINVAL;
    }
    MG_TRY(element_design_only(p, "mg_sensitivity_solve"));
    mg_solve_opts o;
    if (opts) o = *opts; else mg_default_solve_opts(&o);
    double *dX = p->d_tmp;  // the resident solution is left as it is
    MG_TRY(to_device_vec(p, X, dX, p->n_dofs));
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) p->jacobian_valid = false;
    MG_TRY(assemble_system(p, dX, nullptr, true, true));
    MG_TRY(assemble_param_residual(p, dX, kind, index, p->d_R));
    std::vector<double> b(p->n_dofs);
    MG_TRY(to_host_vec(p, p->d_R, b.data(), p->n_dofs));
    for (int64_t i = 0; i < p->n_dofs; i++) b[i] = p->h_fixed[i] ? 0.0 : -b[i];
    MG_TRY(to_device_vec(p, b.data(), p->d_R, p->n_dofs));
    double *dsol = p->d_tmp2;
    MG_CUDA_TRY(cudaMemsetAsync(dsol, 0, p->n_dofs * 8, p->stream));
    int its = 0;
    double rr = 0;
    // the consistent conduction Jacobian is not symmetric: BiCGStab there
    const int kr = p->physics == MG_PHYSICS_HEAT_QUAD4 ? MG_KRYLOV_BICGSTAB : o.krylov;
    MG_TRY(krylov_solve(p, p->A, p->d_R, dsol, o, kr, &its, &rr));
    return to_host_vec(p, dsol, du_dp, p->n_dofs);
}

int mg_output_derivative(mg_problem *p, int32_t output, const double *X, double *dq_dX) {
    // AssemblyBase::calculate_output_derivative (assembly_base.cpp:336-429): dq/dX, zero on
    // constrained dofs
    if (!p || !dq_dX) {
        set_error("mg_output_derivative: invalid argument");
        return MG_EINVAL;
    }
    if (output == MG_OUTPUT_COMPLIANCE) {
        if (p->physics != MG_PHYSICS_ELASTICITY_HEX8 && p->physics != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR &&
            p->physics != MG_PHYSICS_MEMBRANE_QUAD4) {
            set_error("compliance: structural physics only");
            return MG_ENOTSUP;
        }
        // C = F . X with F independent of X: dC/dX = F (the load vector, zero on fixed dofs)
        for (int64_t i = 0; i < p->n_dofs; i++) dq_dX[i] = p->h_F[i];
        return MG_OK;
    }
    if (output == MG_OUTPUT_MEAN_TEMPERATURE) {
        if (p->physics != MG_PHYSICS_HEAT_QUAD4) {
            set_error("mean temperature: heat physics only");
            return MG_ENOTSUP;
        }
        const double *dT = p->d_X;
        if (X) {
            MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
            dT = p->d_tmp;
        }
        double qbar = 0;
        MG_TRY(mean_temperature_terms(p, dT, p->d_R, &qbar));
        MG_TRY(to_host_vec(p, p->d_R, dq_dX, p->n_dofs));
        for (int64_t i = 0; i < p->n_dofs; i++)
            if (p->h_fixed[i]) dq_dX[i] = 0.0;
        return MG_OK;
    }
    set_error("mg_output_derivative: unknown output %d", output);
    return MG_EINVAL;
}

namespace {
// device copies of one element's local vector and matrices for the per-element calls
struct ElemBuffers {
    double *sol = nullptr, *Ke = nullptr, *fe = nullptr;
    int32_t *slot = nullptr;
    ~ElemBuffers() {
        dev_free(sol);
        dev_free(Ke);
        dev_free(fe);
        dev_free(slot);
    }
    int alloc(int nd) {
        MG_TRY(dev_alloc_n(&sol, (size_t)nd));
        MG_TRY(dev_alloc_n(&Ke, (size_t)nd * nd));
        MG_TRY(dev_alloc_n(&fe, (size_t)nd));
        return dev_alloc(reinterpret_cast<void **>(&slot), 64);
    }
};
}  // namespace

int mg_element_calculations(mg_problem *p, int64_t elem, const double *sol_elem, double *Ke,
                            double *fe) {
    if (!p || elem < 0 || elem >= p->n_elems || !sol_elem || (!Ke && !fe)) {
        set_error("mg_element_calculations: invalid argument");
        return MG_EINVAL;
    }
    const int nd = p->npe * p->dpn;
    for (int i = 0; i < nd; i++)
        if (!std::isfinite(sol_elem[i])) {
            set_error("mg_element_calculations: non-finite element solution");
            return MG_EINVAL;
        }
    ElemBuffers b;
    MG_TRY(b.alloc(nd));
    MG_CUDA_TRY(cudaMemcpyAsync(b.sol, sol_elem, nd * 8, cudaMemcpyHostToDevice, p->stream));
    MG_TRY(element_calculations(p, elem, b.sol, b.Ke, b.fe, b.slot));
    if (Ke) MG_CUDA_TRY(cudaMemcpyAsync(Ke, b.Ke, (size_t)nd * nd * 8, cudaMemcpyDeviceToHost, p->stream));
    if (fe) MG_CUDA_TRY(cudaMemcpyAsync(fe, b.fe, (size_t)nd * 8, cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int mg_element_sensitivity(mg_problem *p, int64_t elem, const double *sol_elem, int32_t kind,
                           int64_t index, double *dfe) {
    if (!p || elem < 0 || elem >= p->n_elems || !sol_elem || !dfe) {
        set_error("mg_element_sensitivity: invalid argument");
        return MG_EINVAL;
    }
    MG_TRY(element_design_only(p, "mg_element_sensitivity"));
    const int nd = p->npe * p->dpn;
    ElemBuffers b;
    MG_TRY(b.alloc(nd));
    MG_CUDA_TRY(cudaMemcpyAsync(b.sol, sol_elem, nd * 8, cudaMemcpyHostToDevice, p->stream));
    MG_TRY(element_sensitivity(p, elem, b.sol, kind, index, b.fe));
    MG_CUDA_TRY(cudaMemcpyAsync(dfe, b.fe, (size_t)nd * 8, cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int mg_mean_temperature(mg_problem *p, const double *T, const mg_solve_opts *opts, double *qbar,
                        double *dq_dk0, double *dq_ds) {
    if (!p) return MG_EINVAL;
    if (p->physics != MG_PHYSICS_HEAT_QUAD4) return MG_ENOTSUP;
    mg_solve_opts o;
    if (opts) o = *opts; else mg_default_solve_opts(&o);
    double *dT = p->d_X;
    if (T) {
        MG_TRY(to_device_vec(p, T, p->d_X, p->n_dofs));
    }
    double q = 0;
    // d_R <- dq/dT
    MG_TRY(mean_temperature_terms(p, dT, p->d_R, &q));
    if (qbar) *qbar = q;
    if (!dq_dk0 && !dq_ds) return MG_OK;
    // adjoint J^T lambda = -dq/dT (consistent Jacobian at T)
    p->jacobian_valid = false;
    MG_TRY(assemble_system(p, dT, nullptr, true, true));
    CsrMatrix At;
    MG_TRY(transpose_csr(p, p->A, &At));
    masked_neg_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(p->n_dofs, p->d_R, p->d_fixed, p->d_tmp);
    MG_CUDA_TRY(cudaGetLastError());
    double *lam = p->d_tmp2;
    MG_CUDA_TRY(cudaMemsetAsync(lam, 0, p->n_dofs * 8, p->stream));
    int its = 0;
    double rr = 0;
    int rc = krylov_solve(p, At, p->d_tmp, lam, o, o.krylov, &its, &rr);
    free_csr(&At);
    if (rc != MG_OK) return rc;
    if (dq_dk0) {
        MG_TRY(elem_sensitivity(p, dT, lam, MG_PARAM_K0, p->d_elem_out));
        std::vector<double> h(p->n_elems);
        MG_TRY(to_host_vec(p, p->d_elem_out, h.data(), p->n_elems));
        double s = 0;
        for (double v : h) s += v;
        *dq_dk0 = s;
    }
    if (dq_ds) {
        MG_TRY(elem_sensitivity(p, dT, lam, MG_PARAM_ELEM_SCALE, p->d_elem_out));
        MG_TRY(to_host_vec(p, p->d_elem_out, dq_ds, p->n_elems));
    }
    return MG_OK;
}

long long mg_launch_count(void) { return g_launches.load(); }

int mg_compliance_resident(mg_problem *p, double *compliance) {
    if (!p) return MG_EINVAL;
    MG_TRY(element_design_only(p, "mg_compliance_resident"));
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8) return MG_ENOTSUP;
    if (p->last_solve_mixed) return matfree_compliance_resident(p, compliance);
    if (compliance) MG_TRY(dot(p, p->d_F, p->d_X, p->n_dofs, compliance));
    count_launches(2);
    MG_TRY(elem_sensitivity(p, p->d_X, p->d_X, MG_PARAM_DENSITY, p->d_elem_out));
    count_launches(1);
    return MG_OK;
}

const double *mg_sensitivities_device(mg_problem *p) { return p ? p->d_elem_out : nullptr; }

int mg_debug_launch_assembly(mg_problem *p, const double *X, int reps) {
    if (!p || reps <= 0) return MG_EINVAL;
    if (X) MG_TRY(to_device_vec(p, X, p->d_tmp, p->n_dofs));
    return launch_assembly(p, p->d_tmp, reps);
}

int mg_debug_launch_apply(mg_problem *p, int precision, int reps) {
    if (!p || reps <= 0) return MG_EINVAL;
    if (precision == MG_PLAIN_FP64) return krylov_launch_spmv_cg(p, reps);
    return matfree_launch_apply(p, precision, reps);
}

// Applies the mixed-precision matrix-free operator once (FP32 in/out through
// host FP64 buffers); Dirichlet entries of x must be zero.
int mg_debug_matfree_apply(mg_problem *p, int precision, const double *x, double *y) {
    if (!p || !x || !y) return MG_EINVAL;
    if ((precision < MG_MIXED_TF32 || precision > MG_MIXED_BF16X3) && precision != MG_OPERATOR_FACTORED_FP32)
        return MG_EINVAL;
    return matfree_apply_debug(p, precision, x, y);
}

}  // extern "C"
