// krylov.cu -- FP64 CSR SpMV and Jacobi-preconditioned Krylov solvers (the role
// PETSc KSP plays under libMesh/SNES in NonlinearSystem::solve,
// src/base/nonlinear_system.cpp:209-235).
//
// Layout: node-interleaved CSR (dof = dpn*node + comp).  The dpn rows of a node
// share one column pattern, so the SpMV walks a node's column list once and
// feeds dpn value streams from it: one group of G lanes per node, coalesced
// column/value loads, the x-vector gather shared by the node's rows.
//
// Reductions are deterministic: every kernel that needs a dot product writes
// one partial per block and the last block to finish (threadfence + counter)
// sums the partials in block order and updates the KrylovState scalars the
// next kernel reads.  Iterations run inside captured CUDA graphs; every kernel
// begins with `if (state->done) return`, so a graph holding `chunk`
// iterations overshoots convergence by no-op launches only.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "mg_internal.h"

namespace mg {

namespace {

constexpr int kBS = 256;
// lanes per node in the SpMV: few lanes keep the FP64 work near one FMA per
// stored value (GB300's FP64 rate is the binding limit next to HBM)
constexpr int kSpmvLanes = 4;

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *partials, int stride) {
    __shared__ double sh[NV][kBS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[k][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int i = 0; i < kBS / 32; i++) s += sh[k][i];
            partials[k * stride + blockIdx.x] = s;
        }
    }
}

// returns true in the (single) last block; its threads then see all partials
__device__ __forceinline__ bool last_block(KrylovState *st) {
    __shared__ bool am_last;
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(&st->counter, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return am_last;
}

// fixed-order sum of partials[k*stride + 0..n) by one block
template <int NV>
__device__ __forceinline__ void sum_partials(const double *partials, int stride, int n,
                                             double (&out)[NV]) {
    __shared__ double sh[NV][kBS];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
        for (int i = threadIdx.x; i < n; i += kBS)
            s += __ldcg(partials + k * stride + i);
        sh[k][threadIdx.x] = s;
    }
    __syncthreads();
    for (int width = kBS / 2; width > 0; width >>= 1) {
        if (threadIdx.x < width)
#pragma unroll
            for (int k = 0; k < NV; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + width];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = sh[k][0];
}

__device__ __forceinline__ bool bad(double x) { return !isfinite(x); }

// ---------------------------------------------------------------------------
// SpMV kernels (G lanes per node, DPN rows per node)
// MODE 0: y = A x
// MODE 1: CG: q = A p (x = p), partial0 = p.q, last block: alpha = rz / pq
// MODE 2: BiCGStab v = A y, partial0 = rh.v, last block alpha = rho / (rh.v)
// MODE 3: BiCGStab t = A z, partial0 = t.s, partial1 = t.t, last: omega
// ---------------------------------------------------------------------------
template <int DPN, int G, int MODE>
__global__ void __launch_bounds__(kBS) spmv_kernel(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
    const double *__restrict__ vals, int64_t n_nodes, const double *__restrict__ x,
    const double *__restrict__ z, const double *__restrict__ p_old, double *__restrict__ p_new,
    double *__restrict__ y, const double *__restrict__ aux, KrylovState *st,
    double *__restrict__ partials, int nparts) {
    if (MODE != 0 && st->done) return;
    const int sub = threadIdx.x % G;
    constexpr int kGroupsPerWarp = 32 / G;
    const int64_t warp = ((int64_t)blockIdx.x * kBS + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * kBS >> 5;
    const int gsub = (threadIdx.x & 31) / G;
    double d0 = 0.0, d1 = 0.0;
    // warp-uniform trip count: the group shuffles below need every lane
    for (int64_t base = warp * kGroupsPerWarp; base < n_nodes; base += nwarps * kGroupsPerWarp) {
        const int64_t node = base + gsub;
        const bool valid = node < n_nodes;
        const int64_t r0 = valid ? node * DPN : 0;
        int32_t rp[DPN];
#pragma unroll
        for (int d = 0; d < DPN; d++) rp[d] = __ldg(rowptr + r0 + d);
        const int32_t len = valid ? __ldg(rowptr + r0 + 1) - rp[0] : 0;
        double acc[DPN];
#pragma unroll
        for (int d = 0; d < DPN; d++) acc[d] = 0.0;
        for (int32_t k = sub; k < len; k += G) {
            const int32_t c = __ldg(cols + rp[0] + k);
            const double xc = x[c];
#pragma unroll
            for (int d = 0; d < DPN; d++) acc[d] = fma(__ldg(vals + rp[d] + k), xc, acc[d]);
        }
#pragma unroll
        for (int d = 0; d < DPN; d++)
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o, G);
        if (valid && sub < DPN) {
            double mine = acc[0];
#pragma unroll
            for (int d = 1; d < DPN; d++)
                if (sub == d) mine = acc[d];
            const int64_t row = r0 + sub;
            y[row] = mine;
            if (MODE == 0) {
                d0 = fma(mine, x[row], d0);
            } else if (MODE == 1) {
                d0 = fma(x[row], mine, d0);  // p.q
            } else if (MODE == 2) {
                d0 = fma(aux[row], mine, d0);  // aux = r-hat
            } else {
                d0 = fma(mine, aux[row], d0);  // aux = s
                d1 = fma(mine, mine, d1);
            }
        }
    }
    if (MODE == 0) return;
    double v[2] = {d0, d1};
    block_reduce_store<2>(v, partials, nparts);
    if (!last_block(st)) return;
    double tot[2];
    sum_partials<2>(partials, nparts, gridDim.x, tot);
    if (threadIdx.x == 0) {
        st->counter = 0;
        if (MODE == 1) {
            st->pq = tot[0];
            if (bad(tot[0])) { st->status = MG_ENAN; st->done = 1; }
            else if (!(tot[0] > 0.0)) { st->status = MG_EBREAKDOWN; st->done = 1; }
            else st->alpha = st->rz / tot[0];
        } else if (MODE == 2) {
            st->rv = tot[0];
            if (bad(tot[0])) { st->status = MG_ENAN; st->done = 1; }
            else if (tot[0] == 0.0) { st->status = MG_EBREAKDOWN; st->done = 1; }
            else st->alpha = st->rho / tot[0];
        } else {
            st->ts = tot[0];
            st->tt = tot[1];
            if (bad(tot[0]) || bad(tot[1])) { st->status = MG_ENAN; st->done = 1; }
            else st->omega = (tot[1] > 0.0) ? tot[0] / tot[1] : 0.0;
        }
    }
}

// CG search direction p = z + beta p (its own launch: the SpMV that follows
// reads p at neighbouring rows)
__global__ void __launch_bounds__(kBS) cg_pupdate_kernel(int64_t n, const double *__restrict__ z,
                                                        double *__restrict__ p,
                                                        const KrylovState *st) {
    if (st->done) return;
    const double beta = st->beta;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS)
        p[i] = fma(beta, p[i], z[i]);
}

// CG vector phase: x += alpha p; r -= alpha q; z = D^-1 r; rz, rr -> beta, stop test
__global__ void __launch_bounds__(kBS) cg_update_kernel(int64_t n, double *__restrict__ x,
                                                       double *__restrict__ r,
                                                       double *__restrict__ z,
                                                       const double *__restrict__ p,
                                                       const double *__restrict__ q,
                                                       const double *__restrict__ dinv,
                                                       KrylovState *st,
                                                       double *__restrict__ partials,
                                                       int nparts) {
    if (st->done) return;
    const double alpha = st->alpha;
    double rz = 0.0, rr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS) {
        x[i] = fma(alpha, p[i], x[i]);
        const double ri = fma(-alpha, q[i], r[i]);
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        rz = fma(ri, zi, rz);
        rr = fma(ri, ri, rr);
    }
    double v[2] = {rz, rr};
    block_reduce_store<2>(v, partials, nparts);
    if (!last_block(st)) return;
    double tot[2];
    sum_partials<2>(partials, nparts, gridDim.x, tot);
    if (threadIdx.x == 0) {
        st->counter = 0;
        st->iter += 1;
        st->rr = tot[1];
        if (bad(tot[0]) || bad(tot[1])) {
            st->status = MG_ENAN;
            st->done = 1;
        } else {
            st->beta = tot[0] / st->rz;
            st->rz = tot[0];
            if (tot[1] <= st->tol2) {
                st->done = 1;
            } else if (st->iter >= st->maxit) {
                st->status = MG_ENOCONV;
                st->done = 1;
            }
        }
    }
}

// initial residual: r = b - q (q = A x), z = D^-1 r, p_old = 0; rz, rr, bb
__global__ void __launch_bounds__(kBS) krylov_init_kernel(
    int64_t n, const double *__restrict__ b, const double *__restrict__ q, double *__restrict__ r,
    double *__restrict__ z, double *__restrict__ p_old, double *__restrict__ rh,
    double *__restrict__ v, const double *__restrict__ dinv, KrylovState *st,
    double *__restrict__ partials, int nparts) {
    double rz = 0.0, rr = 0.0, bb = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS) {
        const double ri = b[i] - q[i];
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        p_old[i] = 0.0;
        if (rh) rh[i] = ri;
        if (v) v[i] = 0.0;
        rz = fma(ri, zi, rz);
        rr = fma(ri, ri, rr);
        bb = fma(b[i], b[i], bb);
    }
    double vv[3] = {rz, rr, bb};
    block_reduce_store<3>(vv, partials, nparts);
    if (!last_block(st)) return;
    double tot[3];
    sum_partials<3>(partials, nparts, gridDim.x, tot);
    if (threadIdx.x == 0) {
        st->counter = 0;
        st->rz = tot[0];
        st->rho = tot[1];  // BiCGStab: rh.r with rh = r
        st->rr = tot[1];
        st->bb = tot[2];
        const double bnorm2 = tot[2] > 0.0 ? tot[2] : 1.0;
        st->tol2 = st->tol2 * bnorm2;  // tol2 holds rtol^2 on entry
        st->beta = 0.0;
        st->alpha = 1.0;
        st->omega = 1.0;
        st->iter = 0;
        if (bad(tot[0]) || bad(tot[1]) || bad(tot[2])) {
            st->status = MG_ENAN;
            st->done = 1;
        } else if (tot[1] <= st->tol2) {
            st->done = 1;
        }
    }
}

// BiCGStab: p = r + beta (p - omega v); y = D^-1 p
__global__ void bicg_p_kernel(int64_t n, const double *__restrict__ r, double *__restrict__ p,
                              const double *__restrict__ v, double *__restrict__ y,
                              const double *__restrict__ dinv, const KrylovState *st) {
    if (st->done) return;
    const double beta = st->beta, omega = st->omega;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS) {
        const double pi = fma(beta, fma(-omega, v[i], p[i]), r[i]);
        p[i] = pi;
        y[i] = dinv[i] * pi;
    }
}

// BiCGStab: s = r - alpha v; z = D^-1 s
__global__ void bicg_s_kernel(int64_t n, const double *__restrict__ r, const double *__restrict__ v,
                              double *__restrict__ s, double *__restrict__ z,
                              const double *__restrict__ dinv, const KrylovState *st) {
    if (st->done) return;
    const double alpha = st->alpha;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS) {
        const double si = fma(-alpha, v[i], r[i]);
        s[i] = si;
        z[i] = dinv[i] * si;
    }
}

// BiCGStab: x += alpha y + omega z; r = s - omega t; rho_new = rh.r, rr
__global__ void __launch_bounds__(kBS) bicg_update_kernel(
    int64_t n, double *__restrict__ x, double *__restrict__ r, const double *__restrict__ rh,
    const double *__restrict__ y, const double *__restrict__ z, const double *__restrict__ s,
    const double *__restrict__ t, KrylovState *st, double *__restrict__ partials, int nparts) {
    if (st->done) return;
    const double alpha = st->alpha, omega = st->omega;
    double rhr = 0.0, rr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS) {
        x[i] = fma(omega, z[i], fma(alpha, y[i], x[i]));
        const double ri = fma(-omega, t[i], s[i]);
        r[i] = ri;
        rhr = fma(rh[i], ri, rhr);
        rr = fma(ri, ri, rr);
    }
    double v[2] = {rhr, rr};
    block_reduce_store<2>(v, partials, nparts);
    if (!last_block(st)) return;
    double tot[2];
    sum_partials<2>(partials, nparts, gridDim.x, tot);
    if (threadIdx.x == 0) {
        st->counter = 0;
        st->iter += 1;
        st->rr = tot[1];
        if (bad(tot[0]) || bad(tot[1])) {
            st->status = MG_ENAN;
            st->done = 1;
        } else if (tot[1] <= st->tol2) {
            st->done = 1;
        } else if (st->omega == 0.0 || tot[0] == 0.0) {
            st->status = MG_EBREAKDOWN;
            st->done = 1;
        } else if (st->iter >= st->maxit) {
            st->status = MG_ENOCONV;
            st->done = 1;
        } else {
            st->beta = (tot[0] / st->rho) * (st->alpha / st->omega);
            st->rho = tot[0];
        }
    }
}

__global__ void jacobi_kernel(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                              const double *__restrict__ vals, int64_t n, double *__restrict__ dinv) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (cols[k] == i) d = vals[k];
    dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
}

// two-stage deterministic dot
__global__ void __launch_bounds__(kBS) dot_kernel(const double *__restrict__ a,
                                                 const double *__restrict__ b, int64_t n,
                                                 double *__restrict__ partials) {
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kBS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * kBS)
        s = fma(a[i], b[i], s);
    double v[1] = {s};
    block_reduce_store<1>(v, partials, gridDim.x);
}

__global__ void __launch_bounds__(kBS) sum_kernel(const double *__restrict__ partials, int n,
                                                 double *__restrict__ out) {
    double tot[1];
    sum_partials<1>(partials, n, n, tot);
    if (threadIdx.x == 0) *out = tot[0];
}

// A^T values through the position map of the symmetric pattern
__global__ void tperm_kernel(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                             int64_t n, int32_t *__restrict__ perm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
        int32_t c = cols[k];
        int32_t lo = rowptr[c], hi = rowptr[c + 1] - 1, pos = -1;
        while (lo <= hi) {
            int32_t mid = (lo + hi) >> 1;
            if (cols[mid] == (int32_t)i) { pos = mid; break; }
            if (cols[mid] < (int32_t)i) lo = mid + 1; else hi = mid - 1;
        }
        perm[k] = pos;
    }
}

__global__ void gather_kernel(const double *__restrict__ src, const int32_t *__restrict__ perm,
                              int64_t nnz, double *__restrict__ dst) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) dst[k] = src[perm[k]];
}

inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

__global__ void fill_f64_kernel(double *__restrict__ a, double v, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

template <int MODE>
void launch_spmv(const CsrMatrix &A, cudaStream_t s, int grid, const double *x, const double *z,
                 const double *p_old, double *p_new, double *y, const double *aux,
                 KrylovState *st, double *partials, int nparts) {
    const int64_t nodes = A.n / A.dpn;
    if (A.dpn == 3)
        spmv_kernel<3, kSpmvLanes, MODE><<<grid, kBS, 0, s>>>(A.rowptr, A.cols, A.vals, nodes, x, z,
                                                              p_old, p_new, y, aux, st, partials, nparts);
    else if (A.dpn == 2)
        spmv_kernel<2, kSpmvLanes, MODE><<<grid, kBS, 0, s>>>(A.rowptr, A.cols, A.vals, nodes, x, z,
                                                              p_old, p_new, y, aux, st, partials, nparts);
    else
        spmv_kernel<1, kSpmvLanes, MODE><<<grid, kBS, 0, s>>>(A.rowptr, A.cols, A.vals, nodes, x, z,
                                                              p_old, p_new, y, aux, st, partials, nparts);
}

int spmv_grid(const CsrMatrix &A) {
    const int64_t nodes = A.n / A.dpn;
    const int G = kSpmvLanes;
    int64_t need = (nodes * G + kBS - 1) / kBS;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, 152 * 16));
}

int vec_grid(int64_t n) {
    int64_t need = (n + kBS - 1) / kBS;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, 152 * 8));
}

int read_state(mg_problem *p) {
    KrylovWork &w = p->kw;
    MG_CUDA_TRY(cudaMemcpyAsync(w.state_host, w.state, sizeof(KrylovState), cudaMemcpyDeviceToHost,
                                p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

}  // namespace

int krylov_init(mg_problem *p) {
    KrylovWork &w = p->kw;
    const int64_t n = p->n_dofs;
    w.n = n;
    w.grid = std::max(spmv_grid(p->A), vec_grid(n));
    double **vecs[] = {&w.r, &w.z, &w.p0, &w.p1, &w.q, &w.dinv, &w.rh, &w.v, &w.y, &w.s, &w.t};
    for (double **v : vecs) MG_TRY(dev_alloc_n(v, (size_t)n));
    MG_TRY(dev_alloc_n(&w.partials, (size_t)3 * w.grid));
    MG_TRY(dev_alloc(reinterpret_cast<void **>(&w.state), sizeof(KrylovState)));
    MG_CUDA_TRY(cudaMallocHost(reinterpret_cast<void **>(&w.state_host), sizeof(KrylovState)));
    MG_CUDA_TRY(cudaMemsetAsync(w.state, 0, sizeof(KrylovState), p->stream));
    return MG_OK;
}

void krylov_free(mg_problem *p) {
    KrylovWork &w = p->kw;
    double *vecs[] = {w.r, w.z, w.p0, w.p1, w.q, w.dinv, w.rh, w.v, w.y, w.s, w.t, w.partials};
    for (double *v : vecs) dev_free(v);
    dev_free(w.state);
    if (w.state_host) cudaFreeHost(w.state_host);
    for (auto &g : w.graph_cg)
        if (g) cudaGraphExecDestroy(g);
    if (w.graph_bicg) cudaGraphExecDestroy(w.graph_bicg);
    w = KrylovWork();
}

int spmv(mg_problem *p, const CsrMatrix &A, const double *d_x, double *d_y) {
    launch_spmv<0>(A, p->stream, spmv_grid(A), d_x, nullptr, nullptr, nullptr, d_y, nullptr, nullptr,
                   nullptr, 0);
    MG_CUDA_TRY(cudaGetLastError());
    return MG_OK;
}

int dot(mg_problem *p, const double *a, const double *b, int64_t n, double *out) {
    int grid = vec_grid(n);
    double *partials = p->d_red;  // >= red_blocks doubles
    grid = std::min(grid, p->red_blocks);
    dot_kernel<<<grid, kBS, 0, p->stream>>>(a, b, n, partials);
    MG_CUDA_TRY(cudaGetLastError());
    double *res = p->d_red + p->red_blocks;
    sum_kernel<<<1, kBS, 0, p->stream>>>(partials, grid, res);
    MG_CUDA_TRY(cudaGetLastError());
    MG_CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int transpose_csr(mg_problem *p, const CsrMatrix &A, CsrMatrix *At) {
    // the assembled pattern is structurally symmetric: A^T shares rowptr/cols
    At->n = A.n;
    At->nnz = A.nnz;
    At->dpn = A.dpn;
    int32_t *perm = nullptr;
    MG_TRY(dev_alloc_n(&perm, (size_t)A.nnz));
    MG_TRY(dev_alloc_n(&At->vals, (size_t)A.nnz));
    At->rowptr = A.rowptr;
    At->cols = A.cols;
    tperm_kernel<<<blocks_for(A.n, 128), 128, 0, p->stream>>>(A.rowptr, A.cols, A.n, perm);
    gather_kernel<<<blocks_for(A.nnz, 256), 256, 0, p->stream>>>(A.vals, perm, A.nnz, At->vals);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(p->stream);
    dev_free(perm);
    if (e != cudaSuccess) {
        set_error("transpose: %s", cudaGetErrorString(e));
        return MG_ECUDA;
    }
    return MG_OK;
}

// enqueue `reps` CG SpMV launches q = A p (timing hook; state reset, no sync)
int krylov_launch_spmv_cg(mg_problem *p, int reps) {
    if (!p->jacobian_valid) MG_TRY(assemble_system(p, p->d_X, nullptr, true, false));
    KrylovWork &w = p->kw;
    KrylovState init{};
    init.maxit = 1 << 30;
    MG_CUDA_TRY(cudaMemcpyAsync(w.state, &init, sizeof(KrylovState), cudaMemcpyHostToDevice, p->stream));
    // nonzero search direction so that every timed launch does the full work
    fill_f64_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(w.z, 1.0, p->n_dofs);
    const int sg = spmv_grid(p->A);
    for (int i = 0; i < reps; i++)
        launch_spmv<1>(p->A, p->stream, sg, w.z, nullptr, nullptr, nullptr, w.q, nullptr, w.state,
                       w.partials, w.grid);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(reps);
    return MG_OK;
}

void free_csr(CsrMatrix *A) {
    // only the values are owned by a transposed view
    dev_free(A->vals);
    A->vals = nullptr;
}

// Solve A x = b (x holds the initial guess) with Jacobi-preconditioned CG or
// BiCGStab to ||b - A x|| <= rtol ||b||.  Returns MG_OK, MG_ENOCONV,
// MG_EBREAKDOWN, MG_ENAN or MG_ETIMEDOUT.
int krylov_solve(mg_problem *p, const CsrMatrix &A, const double *d_b, double *d_x,
                 const mg_solve_opts &o, int krylov, int *iters, double *relres) {
    KrylovWork &w = p->kw;
    const int64_t n = A.n;
    cudaStream_t s = p->stream;
    const int sg = spmv_grid(A), vg = vec_grid(n);
    const int nparts = w.grid;
    jacobi_kernel<<<blocks_for(n, 256), 256, 0, s>>>(A.rowptr, A.cols, A.vals, n, w.dinv);
    MG_CUDA_TRY(cudaGetLastError());
    KrylovState init{};
    init.tol2 = o.rtol * o.rtol;
    init.maxit = o.max_iterations > 0 ? o.max_iterations : 100000;
    MG_CUDA_TRY(cudaMemcpyAsync(w.state, &init, sizeof(KrylovState), cudaMemcpyHostToDevice, s));
    MG_TRY(spmv(p, A, d_x, w.q));
    krylov_init_kernel<<<vg, kBS, 0, s>>>(n, d_b, w.q, w.r, w.z, w.p0, w.rh, w.v, w.dinv, w.state,
                                         w.partials, nparts);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(3);
    // CG: p0 = 0 and beta = 0, so the first p update forms p = z
    const int chunk = o.graph_chunk > 0 ? o.graph_chunk : 16;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < chunk; it++) {
        if (krylov == MG_KRYLOV_CG) {
            cg_pupdate_kernel<<<vg, kBS, 0, s>>>(n, w.z, w.p0, w.state);
            launch_spmv<1>(A, s, sg, w.p0, nullptr, nullptr, nullptr, w.q, nullptr, w.state,
                           w.partials, nparts);
            cg_update_kernel<<<vg, kBS, 0, s>>>(n, d_x, w.r, w.z, w.p0, w.q, w.dinv, w.state,
                                                w.partials, nparts);
        } else {
            bicg_p_kernel<<<vg, kBS, 0, s>>>(n, w.r, w.p0, w.v, w.y, w.dinv, w.state);
            launch_spmv<2>(A, s, sg, w.y, nullptr, nullptr, nullptr, w.v, w.rh, w.state, w.partials,
                           nparts);
            bicg_s_kernel<<<vg, kBS, 0, s>>>(n, w.r, w.v, w.s, w.z, w.dinv, w.state);
            launch_spmv<3>(A, s, sg, w.z, nullptr, nullptr, nullptr, w.t, w.s, w.state, w.partials,
                           nparts);
            bicg_update_kernel<<<vg, kBS, 0, s>>>(n, d_x, w.r, w.rh, w.y, w.z, w.s, w.t, w.state,
                                                  w.partials, nparts);
        }
    }
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) {
        set_error("graph capture: %s", cudaGetErrorString(ce));
        return MG_ECUDA;
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        set_error("graph instantiate: %s", cudaGetErrorString(ce));
        return MG_ECUDA;
    }
    const double t0 = wall_time();
    int rc = MG_OK;
    for (;;) {
        rc = read_state(p);
        if (rc != MG_OK) break;
        if (w.state_host->done) break;
        if (o.timeout_s > 0 && wall_time() - t0 > o.timeout_s) {
            rc = MG_ETIMEDOUT;
            set_error("Krylov solve exceeded %.1f s", o.timeout_s);
            break;
        }
        ce = cudaGraphLaunch(exec, s);
        count_launches((long long)chunk * (krylov == MG_KRYLOV_CG ? 3 : 5));
        if (ce != cudaSuccess) {
            set_error("graph launch: %s", cudaGetErrorString(ce));
            rc = MG_ECUDA;
            break;
        }
    }
    cudaGraphExecDestroy(exec);
    if (rc != MG_OK) return rc;
    const KrylovState &h = *w.state_host;
    if (iters) *iters = h.iter;
    if (relres) *relres = (h.bb > 0 ? sqrt(h.rr / h.bb) : sqrt(h.rr));
    return h.status;
}

}  // namespace mg

// ---------------------------------------------------------------------------
// Allocation-free Jacobi-PCG on a caller-owned CSR (mg_pcg_csr_static).
//
// The solver scratch (r, z, the search direction p, A p, the Jacobi inverse,
// the per-block partial sums and the solver state) lives in the file-scope
// device array below instead of memory from cudaMalloc.  Every GPU that loads
// this library holds the array (about 5.3 MB) until the process exits.  All
// calls on a device share it and it keeps the last call's contents, so each
// call re-initialises what must start at zero; calls that overlap on the GPU
// (different streams or threads) race on it.
// ---------------------------------------------------------------------------
namespace mg {
namespace {

constexpr int64_t kStaticMaxN = MG_STATIC_PCG_MAX_N;
constexpr int64_t kStaticVectors = 5;           // r, z, p, q = A p, D^-1
constexpr int64_t kStaticParts = 3 * 152 * 16;  // 3 x the largest grid of the kernels
constexpr int64_t kStaticStateDoubles = 32;     // >= sizeof(KrylovState) / 8
static_assert(sizeof(KrylovState) <= kStaticStateDoubles * sizeof(double), "state slot");

static __device__ __align__(256) double g_static_pcg_scratch[kStaticVectors * kStaticMaxN +
                                                            kStaticParts + kStaticStateDoubles];

// Device address of the static array in the current device's context.  It is
// looked up on every call rather than cached per device ordinal: after a
// cudaDeviceReset, or under another context of the same device, the module is
// loaded again at another address.  The lookup costs microseconds against a
// solve that synchronises its stream every 16 iterations.
int static_scratch(double **out) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_pcg_scratch);
    if (e != cudaSuccess || !ptr) {
        set_error("cudaGetSymbolAddress(static PCG scratch): %s", cudaGetErrorString(e));
        return MG_ECUDA;
    }
    *out = static_cast<double *>(ptr);
    return MG_OK;
}

}  // namespace
}  // namespace mg

extern "C" int mg_pcg_csr_static(int64_t n, const int32_t *rowptr, const int32_t *cols,
                                 const double *vals, const double *b, double *x, double rtol,
                                 int32_t max_iterations, void *stream, int32_t *iterations,
                                 double *relres) {
    using namespace mg;
    if (n <= 0 || !rowptr || !cols || !vals || !b || !x || !(rtol > 0.0)) {
        set_error("mg_pcg_csr_static: invalid argument");
        return MG_EINVAL;
    }
    if (n > kStaticMaxN) {
        set_error("mg_pcg_csr_static: n = %lld exceeds the static scratch limit of %lld dofs "
                  "(MG_STATIC_PCG_MAX_N)", (long long)n, (long long)kStaticMaxN);
        return MG_EINVAL;
    }
    double *base = nullptr;
    MG_TRY(static_scratch(&base));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *r = base, *z = base + kStaticMaxN, *p0 = base + 2 * kStaticMaxN,
           *q = base + 3 * kStaticMaxN, *dinv = base + 4 * kStaticMaxN,
           *partials = base + kStaticVectors * kStaticMaxN;
    KrylovState *state =
        reinterpret_cast<KrylovState *>(base + kStaticVectors * kStaticMaxN + kStaticParts);
    CsrMatrix A;
    A.n = n;
    A.nnz = 0;
    A.dpn = 1;  // general CSR: one row per group of lanes
    A.rowptr = const_cast<int32_t *>(rowptr);
    A.cols = const_cast<int32_t *>(cols);
    A.vals = const_cast<double *>(vals);
    const int sg = spmv_grid(A), vg = vec_grid(n);
    const int nparts = std::max(sg, vg);
    jacobi_kernel<<<blocks_for(n, 256), 256, 0, s>>>(rowptr, cols, vals, n, dinv);
    KrylovState init{};
    init.tol2 = rtol * rtol;
    init.maxit = max_iterations > 0 ? max_iterations : 100000;
    MG_CUDA_TRY(cudaMemcpyAsync(state, &init, sizeof(KrylovState), cudaMemcpyHostToDevice, s));
    launch_spmv<0>(A, s, sg, x, nullptr, nullptr, nullptr, q, nullptr, nullptr, nullptr, 0);
    krylov_init_kernel<<<vg, kBS, 0, s>>>(n, b, q, r, z, p0, nullptr, nullptr, dinv, state,
                                         partials, nparts);
    MG_CUDA_TRY(cudaGetLastError());
    KrylovState h{};
    for (;;) {
        MG_CUDA_TRY(cudaMemcpyAsync(&h, state, sizeof(KrylovState), cudaMemcpyDeviceToHost, s));
        MG_CUDA_TRY(cudaStreamSynchronize(s));
        if (h.done) break;
        for (int it = 0; it < 16; it++) {
            cg_pupdate_kernel<<<vg, kBS, 0, s>>>(n, z, p0, state);
            launch_spmv<1>(A, s, sg, p0, nullptr, nullptr, nullptr, q, nullptr, state, partials,
                           nparts);
            cg_update_kernel<<<vg, kBS, 0, s>>>(n, x, r, z, p0, q, dinv, state, partials, nparts);
        }
        MG_CUDA_TRY(cudaGetLastError());
        count_launches(48);
    }
    if (iterations) *iterations = h.iter;
    if (relres) *relres = h.bb > 0 ? sqrt(h.rr / h.bb) : sqrt(h.rr);
    return h.status;
}

