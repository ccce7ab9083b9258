// filter.cu -- the density filter of MAST::FilterBase on the GPU (mg_filter_*).
//
// MAST (src/level_set/filter_base.cpp) filters the design field with
// normalised hat weights: point i takes w_ij = (r - d_ij) / sum_k (r - d_ik)
// over all points j within distance r (`_init` :378-437, `_init2` :275-359);
// compute_filtered_values (:58-95) forms sum_j w_ij x_j for design-variable
// points and passes the others through.  The design-gradient chain rule of the
// topology-optimisation loop (examples/structural/example_6/example_6.cpp:
// 661-697, where the filtered unit perturbations become the density
// sensitivities) is the transpose: dq/dx = F^T dq/dx_filtered.
//
// Two layouts:
//   * structured grids: the element centroids form a lattice, so the weights
//     are one stencil of integer offsets; a kernel applies it with the per-point
//     normalisation (which only differs near the boundary) precomputed;
//   * arbitrary points: the neighbour lists are found on the host with a
//     bucket grid of cell size r and stored as a CSR matrix and its transpose;
//     FP64 CSR products apply F and F^T.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <unordered_map>
#include <vector>

#include "mg_internal.h"

namespace mg {
namespace {

inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

struct StencilArgs {
    int nx, ny, nz;       // grid (nz = 1 in 2D)
    int n_off;
    const int *ox, *oy, *oz;
    const double *w;      // r - d per offset
};

// S_e = sum of the in-domain stencil weights; stores 1 / S_e
__global__ void stencil_norm_kernel(StencilArgs a, double *__restrict__ inv_s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % a.nx), j = (int)((e / a.nx) % a.ny), k = (int)(e / ((int64_t)a.nx * a.ny));
        double s = 0.0;
        for (int o = 0; o < a.n_off; o++) {
            const int ii = i + a.ox[o], jj = j + a.oy[o], kk = k + a.oz[o];
            if (ii < 0 || jj < 0 || kk < 0 || ii >= a.nx || jj >= a.ny || kk >= a.nz) continue;
            s += a.w[o];
        }
        inv_s[e] = 1.0 / s;
    }
}

// forward: out_e = dv_e ? sum_o w_o in_{e+o} / S_e : in_e
// transpose: out_f = (dv_f ? 0 : in_f) + sum_o w_o [dv_{f+o}] in_{f+o} / S_{f+o}
// (the stencil is symmetric, so the transpose gathers over the same offsets)
__global__ void stencil_apply_kernel(StencilArgs a, const double *__restrict__ inv_s,
                                     const uint8_t *__restrict__ dv, const double *__restrict__ in,
                                     double *__restrict__ out, int transpose) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % a.nx), j = (int)((e / a.nx) % a.ny), k = (int)(e / ((int64_t)a.nx * a.ny));
        const bool is_dv = !dv || dv[e];
        if (!transpose && !is_dv) {
            out[e] = in[e];
            continue;
        }
        double acc = 0.0;
        for (int o = 0; o < a.n_off; o++) {
            const int ii = i + a.ox[o], jj = j + a.oy[o], kk = k + a.oz[o];
            if (ii < 0 || jj < 0 || kk < 0 || ii >= a.nx || jj >= a.ny || kk >= a.nz) continue;
            const int64_t f = ii + (int64_t)a.nx * (jj + (int64_t)a.ny * kk);
            if (!transpose) acc = fma(a.w[o], in[f], acc);
            else if (!dv || dv[f]) acc = fma(a.w[o], in[f] * inv_s[f], acc);
        }
        out[e] = transpose ? (is_dv ? acc : acc + in[e]) : acc * inv_s[e];
    }
}

// y_i = (pass_i ? x_i : 0) + sum_k vals_k x_cols_k (one warp per row)
__global__ void csr_filter_kernel(int64_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                  const double *__restrict__ vals, const uint8_t *__restrict__ pass,
                                  const uint8_t *__restrict__ gate, const double *__restrict__ x,
                                  double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n;
         row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        double acc = 0.0;
        for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) {
            const int32_t c = cols[k];
            if (!gate || gate[c]) acc = fma(vals[k], x[c], acc);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) y[row] = (pass && pass[row]) ? x[row] + acc : acc;
    }
}

}  // namespace
}  // namespace mg

using namespace mg;

struct mg_filter {
    cudaStream_t stream = nullptr;
    int64_t n = 0, nnz = 0;
    bool grid = false;
    StencilArgs st{};
    int *d_ox = nullptr, *d_oy = nullptr, *d_oz = nullptr;
    double *d_w = nullptr, *d_inv_s = nullptr;
    uint8_t *d_dv = nullptr, *d_not_dv = nullptr;
    // points: F (rows: filtered points) and F^T, normalised weights
    int64_t *d_rp = nullptr, *d_rpt = nullptr;
    int32_t *d_c = nullptr, *d_ct = nullptr;
    double *d_v = nullptr, *d_vt = nullptr;
    double *d_in = nullptr, *d_out = nullptr;  // staging for host buffers
};

namespace mg {
namespace {

template <class T>
int upload(T **dst, const T *src, size_t n, cudaStream_t s) {
    MG_TRY(dev_alloc_n(dst, std::max<size_t>(n, 1)));
    if (n) MG_CUDA_TRY(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return MG_OK;
}

int finish_create(mg_filter *f, const uint8_t *dv) {
    MG_TRY(dev_alloc_n(&f->d_in, (size_t)f->n));
    MG_TRY(dev_alloc_n(&f->d_out, (size_t)f->n));
    if (dv) {
        MG_TRY(upload(&f->d_dv, dv, (size_t)f->n, f->stream));
        std::vector<uint8_t> nd((size_t)f->n);
        for (int64_t i = 0; i < f->n; i++) nd[i] = dv[i] ? 0 : 1;
        MG_TRY(upload(&f->d_not_dv, nd.data(), nd.size(), f->stream));
        MG_CUDA_TRY(cudaStreamSynchronize(f->stream));
    }
    return MG_OK;
}

int run(mg_filter *f, const double *in, double *out, int transpose, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        MG_CUDA_TRY(cudaGetDevice(&dev));
        MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    if (f->grid) {
        const unsigned g = std::min(blocks_for(f->n, 256), (unsigned)(8 * sms));
        stencil_apply_kernel<<<g, 256, 0, s>>>(f->st, f->d_inv_s, f->d_dv, in, out, transpose);
    } else {
        const unsigned g = std::min(blocks_for(f->n * 32, 256), 65535u);
        // F holds unit rows for non-design points; F^T holds the design rows'
        // entries only, plus the pass-through of non-design points
        if (!transpose)
            csr_filter_kernel<<<g, 256, 0, s>>>(f->n, f->d_rp, f->d_c, f->d_v, nullptr, nullptr, in, out);
        else
            csr_filter_kernel<<<g, 256, 0, s>>>(f->n, f->d_rpt, f->d_ct, f->d_vt, f->d_not_dv, nullptr, in, out);
    }
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return MG_OK;
}

}  // namespace
}  // namespace mg

extern "C" {

int mg_filter_create_grid(int32_t nx, int32_t ny, int32_t nz, double hx, double hy, double hz, double radius,
                          const uint8_t *dv_mask, mg_filter **out) {
    if (!out) return MG_EINVAL;
    *out = nullptr;
    const int NZ = nz > 0 ? nz : 1;
    if (nx <= 0 || ny <= 0 || nz < 0 || !(radius > 0.0) || !(hx > 0.0) || !(hy > 0.0) || (nz > 0 && !(hz > 0.0))) {
        set_error("mg_filter_create_grid: bad grid or radius");
        return MG_EINVAL;
    }
    // stencil: integer offsets within the radius (weight r - d, 0 at d = r kept out)
    std::vector<int> ox, oy, oz;
    std::vector<double> w;
    const int ax = (int)floor(radius / hx), ay = (int)floor(radius / hy), az = nz > 0 ? (int)floor(radius / hz) : 0;
    if ((int64_t)(2 * ax + 1) * (2 * ay + 1) * (2 * az + 1) > 1 << 20) {
        set_error("mg_filter_create_grid: radius spans too many elements");
        return MG_EINVAL;
    }
    for (int c = -az; c <= az; c++)
        for (int b = -ay; b <= ay; b++)
            for (int a = -ax; a <= ax; a++) {
                const double d = sqrt((a * hx) * (a * hx) + (b * hy) * (b * hy) + (c * hz) * (c * hz));
                if (d <= radius && radius - d > 0.0) {
                    ox.push_back(a);
                    oy.push_back(b);
                    oz.push_back(c);
                    w.push_back(radius - d);
                }
            }
    mg_filter *f = new mg_filter();
    auto fail = [&](int rc) {
        mg_filter_destroy(f);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete f;
        set_error("cudaStreamCreate failed (no usable GPU?)");
        return MG_ECUDA;
    }
    f->grid = true;
    f->n = (int64_t)nx * ny * NZ;
    f->nnz = (int64_t)w.size();
    int rc;
    if ((rc = upload(&f->d_ox, ox.data(), ox.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_oy, oy.data(), oy.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_oz, oz.data(), oz.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_w, w.data(), w.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = dev_alloc_n(&f->d_inv_s, (size_t)f->n)) != MG_OK) return fail(rc);
    f->st = StencilArgs{nx, ny, NZ, (int)w.size(), f->d_ox, f->d_oy, f->d_oz, f->d_w};
    stencil_norm_kernel<<<std::min(blocks_for(f->n, 256), 4096u), 256, 0, f->stream>>>(f->st, f->d_inv_s);
    count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return fail(MG_ECUDA);
    if ((rc = finish_create(f, dv_mask)) != MG_OK) return fail(rc);
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return fail(MG_ECUDA);
    *out = f;
    return MG_OK;
}

int mg_filter_create_points(int64_t n, int32_t dim, const double *xyz, double radius, const uint8_t *dv_mask,
                            mg_filter **out) {
    if (!out) return MG_EINVAL;
    *out = nullptr;
    if (n <= 0 || n > INT32_MAX || dim < 1 || dim > 3 || !xyz || !(radius > 0.0)) {
        set_error("mg_filter_create_points: bad points or radius");
        return MG_EINVAL;
    }
    for (int64_t i = 0; i < n * dim; i++)
        if (!isfinite(xyz[i])) {
            set_error("mg_filter_create_points: non-finite coordinate");
            return MG_EINVAL;
        }
    // bucket grid of cell size r: neighbours lie in the 3^dim surrounding cells
    double lo[3] = {0, 0, 0};
    for (int c = 0; c < dim; c++) {
        lo[c] = xyz[c];
        for (int64_t i = 0; i < n; i++) lo[c] = std::min(lo[c], xyz[i * dim + c]);
    }
    auto cell_of = [&](int64_t i, int c) { return (int64_t)floor((xyz[i * dim + c] - lo[c]) / radius); };
    auto key = [](int64_t a, int64_t b, int64_t c) { return (a * 73856093LL) ^ (b * 19349663LL) ^ (c * 83492791LL); };
    std::unordered_map<int64_t, std::vector<int32_t>> buckets;
    buckets.reserve((size_t)n);
    for (int64_t i = 0; i < n; i++)
        buckets[key(cell_of(i, 0), dim > 1 ? cell_of(i, 1) : 0, dim > 2 ? cell_of(i, 2) : 0)].push_back((int32_t)i);
    std::vector<int64_t> rp((size_t)n + 1, 0);
    std::vector<int32_t> cols;
    std::vector<double> vals;
    std::vector<std::pair<int32_t, double>> row;
    for (int64_t i = 0; i < n; i++) {
        row.clear();
        const int64_t ci = cell_of(i, 0), cj = dim > 1 ? cell_of(i, 1) : 0, ck = dim > 2 ? cell_of(i, 2) : 0;
        double sum = 0.0;
        for (int64_t dk = (dim > 2 ? -1 : 0); dk <= (dim > 2 ? 1 : 0); dk++)
            for (int64_t dj = (dim > 1 ? -1 : 0); dj <= (dim > 1 ? 1 : 0); dj++)
                for (int64_t di = -1; di <= 1; di++) {
                    auto it = buckets.find(key(ci + di, cj + dj, ck + dk));
                    if (it == buckets.end()) continue;
                    for (int32_t j : it->second) {
                        double d2 = 0.0;
                        for (int c = 0; c < dim; c++) {
                            const double t = xyz[i * dim + c] - xyz[(int64_t)j * dim + c];
                            d2 += t * t;
                        }
                        const double d = sqrt(d2);
                        if (d <= radius && radius - d > 0.0) {
                            row.push_back({j, radius - d});
                            sum += radius - d;
                        }
                    }
                }
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end(),
                              [](const std::pair<int32_t, double> &a, const std::pair<int32_t, double> &b) {
                                  return a.first == b.first;
                              }),
                  row.end());
        // recompute the sum over the unique neighbours (hash collisions may repeat a bucket)
        sum = 0.0;
        for (auto &p : row) sum += p.second;
        const bool is_dv = !dv_mask || dv_mask[i];
        if (is_dv)
            for (auto &p : row) {
                cols.push_back(p.first);
                vals.push_back(p.second / sum);
            }
        else {  // a non-design point keeps its value: unit row
            cols.push_back((int32_t)i);
            vals.push_back(1.0);
        }
        rp[i + 1] = (int64_t)cols.size();
    }
    // F^T restricted to design rows (the non-design identity is added by the kernel)
    std::vector<int64_t> rpt((size_t)n + 1, 0);
    std::vector<int64_t> cnt((size_t)n, 0);
    for (int64_t i = 0; i < n; i++)
        if (!dv_mask || dv_mask[i])
            for (int64_t k = rp[i]; k < rp[i + 1]; k++) cnt[cols[k]]++;
    for (int64_t j = 0; j < n; j++) rpt[j + 1] = rpt[j] + cnt[j];
    std::vector<int32_t> ct((size_t)rpt[n]);
    std::vector<double> vt((size_t)rpt[n]);
    std::vector<int64_t> pos(rpt.begin(), rpt.end() - 1);
    for (int64_t i = 0; i < n; i++)
        if (!dv_mask || dv_mask[i])
            for (int64_t k = rp[i]; k < rp[i + 1]; k++) {
                const int64_t p = pos[cols[k]]++;
                ct[p] = (int32_t)i;
                vt[p] = vals[k];
            }
    mg_filter *f = new mg_filter();
    auto fail = [&](int rc) {
        mg_filter_destroy(f);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete f;
        set_error("cudaStreamCreate failed (no usable GPU?)");
        return MG_ECUDA;
    }
    f->n = n;
    f->nnz = (int64_t)cols.size();
    int rc;
    if ((rc = upload(&f->d_rp, rp.data(), rp.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_c, cols.data(), cols.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_v, vals.data(), vals.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_rpt, rpt.data(), rpt.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_ct, ct.data(), ct.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = upload(&f->d_vt, vt.data(), vt.size(), f->stream)) != MG_OK) return fail(rc);
    if ((rc = finish_create(f, dv_mask)) != MG_OK) return fail(rc);
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return fail(MG_ECUDA);
    *out = f;
    return MG_OK;
}

int mg_filter_info(const mg_filter *f, int64_t *n, int64_t *nnz) {
    if (!f) return MG_EINVAL;
    if (n) *n = f->n;
    if (nnz) *nnz = f->nnz;
    return MG_OK;
}

int mg_filter_apply_device(mg_filter *f, const double *in_dev, double *out_dev, int32_t transpose, void *stream) {
    if (!f || !in_dev || !out_dev || in_dev == out_dev) return MG_EINVAL;
    cudaStream_t s = stream ? (cudaStream_t)stream : f->stream;
    return run(f, in_dev, out_dev, transpose, s);
}

int mg_filter_apply(mg_filter *f, const double *in, double *out, int32_t transpose) {
    if (!f || !in || !out) return MG_EINVAL;
    MG_CUDA_TRY(cudaMemcpyAsync(f->d_in, in, f->n * 8, cudaMemcpyHostToDevice, f->stream));
    MG_TRY(run(f, f->d_in, f->d_out, transpose, f->stream));
    MG_CUDA_TRY(cudaMemcpyAsync(out, f->d_out, f->n * 8, cudaMemcpyDeviceToHost, f->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(f->stream));
    return MG_OK;
}

void mg_filter_destroy(mg_filter *f) {
    if (!f) return;
    if (f->stream) cudaStreamSynchronize(f->stream);
    void *p[] = {f->d_ox, f->d_oy, f->d_oz, f->d_w, f->d_inv_s, f->d_dv, f->d_not_dv, f->d_rp, f->d_rpt,
                 f->d_c, f->d_ct, f->d_v, f->d_vt, f->d_in, f->d_out};
    for (void *q : p) dev_free(q);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
}

}  // extern "C"
