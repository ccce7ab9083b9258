// assembly.cu -- FP64 element quadrature kernels and the coloured, atomic-free
// scatter into the device CSR (plain form of the MAST hot path).
//
// HEX8 elasticity restates StructuralElement3D::internal_residual
// (src/elasticity/solid_element_3d.cpp:135-423, linear-strain branch) with the
// isotropic material of IsotropicMaterialProperty::StiffnessMatrix3D
// (src/property_cards/isotropic_material_property_card.cpp:512-528).  For an
// element-constant isotropic C the (a,b) 3x3 block of sum_qp JxW B^T C B is
//     lambda S + mu S^T + mu tr(S) I,   S_ij = sum_qp JxW dphi_a/dx_i dphi_b/dx_j,
// the same integral evaluated with 9 instead of 6*6*24*2 products per pair and
// quadrature point.  Blocks are emitted in MAST's variable-blocked element order
// (src/numerics/fem_operator_matrix.h:262-300) when element matrices are
// requested, and scattered into the node-interleaved CSR otherwise.
#include <cuda_runtime.h>
#include <math.h>

#include "hex8_gl.cuh"
#include "side_loads.cuh"
#include "mg_internal.h"

namespace mg {

namespace {

constexpr double kGP = 0.57735026918962576451;  // 1/sqrt(3)

__device__ __forceinline__ double gauss_coord(int bit) { return bit ? kGP : -kGP; }

// libMesh HEX8 node signs (ext.)
__device__ __forceinline__ void hex8_sign(int a, double &sx, double &sy, double &sz) {
    sx = ((a + 1) >> 1 & 1) ? 1.0 : -1.0;  // 0:-,1:+,2:+,3:-
    sy = (a >> 1 & 1) ? 1.0 : -1.0;        // 0:-,1:-,2:+,3:+
    sz = (a >> 2 & 1) ? 1.0 : -1.0;
}

// reference gradient d phi_a / d xi_i at Gauss point q (q = i + 2j + 4k)
__device__ __forceinline__ void hex8_dref(int q, int a, double d[3]) {
    double xi = gauss_coord(q & 1), eta = gauss_coord(q >> 1 & 1), zeta = gauss_coord(q >> 2 & 1);
    double sx, sy, sz;
    hex8_sign(a, sx, sy, sz);
    double fx = 0.5 * (1.0 + sx * xi), fy = 0.5 * (1.0 + sy * eta), fz = 0.5 * (1.0 + sz * zeta);
    d[0] = 0.5 * sx * fy * fz;
    d[1] = 0.5 * sy * fx * fz;
    d[2] = 0.5 * sz * fx * fy;
}

__device__ __forceinline__ void quad4_sign(int a, double &sx, double &sy) {
    sx = ((a + 1) >> 1 & 1) ? 1.0 : -1.0;
    sy = (a >> 1 & 1) ? 1.0 : -1.0;
}

// QUAD4 shape data at Gauss point q: phi, physical gradient, JxW
__device__ __forceinline__ double quad4_qp(const double X[8], int q, double phi[4],
                                           double g[8]) {
    double xi = gauss_coord(q & 1), eta = gauss_coord(q >> 1 & 1);
    double dref[8];
    for (int a = 0; a < 4; a++) {
        double sx, sy;
        quad4_sign(a, sx, sy);
        double fx = 0.5 * (1.0 + sx * xi), fy = 0.5 * (1.0 + sy * eta);
        phi[a] = fx * fy;
        dref[a * 2 + 0] = 0.5 * sx * fy;
        dref[a * 2 + 1] = 0.5 * sy * fx;
    }
    double J0 = 0, J1 = 0, J2 = 0, J3 = 0;
    for (int a = 0; a < 4; a++) {
        J0 += dref[a * 2] * X[a * 2];
        J1 += dref[a * 2] * X[a * 2 + 1];
        J2 += dref[a * 2 + 1] * X[a * 2];
        J3 += dref[a * 2 + 1] * X[a * 2 + 1];
    }
    double det = J0 * J3 - J1 * J2;
    double i0 = J3 / det, i1 = -J1 / det, i2 = -J2 / det, i3 = J0 / det;
    for (int a = 0; a < 4; a++) {
        g[a * 2 + 0] = i0 * dref[a * 2] + i1 * dref[a * 2 + 1];
        g[a * 2 + 1] = i2 * dref[a * 2] + i3 * dref[a * 2 + 1];
    }
    return det;  // weight 1 for the 2-point rule
}

constexpr int kWarpsPerBlock = 8;

// ---------------------------------------------------------------------------
// HEX8: one warp per element.  MODE 0: scatter into CSR; MODE 1: write the
// 24x24 element matrix (var-blocked); MODE 2: per-element bilinear form
// out[e] = scale_e * a_e^T K1_e b_e (K1 = stiffness at E = 1).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) hex8_kernel(
    const double *__restrict__ coords, const int32_t *__restrict__ conn,
    const int32_t *__restrict__ elem_list, int64_t first, int64_t n_items,
    const double *__restrict__ E_elem, const double *__restrict__ E_qp, double lam1, double mu1,
    const int32_t *__restrict__ rowptr, const uint16_t *__restrict__ emap,
    double *__restrict__ vals, double *__restrict__ Ke_out,
    const double *__restrict__ va, const double *__restrict__ vb,
    const uint8_t *__restrict__ fixed, double *__restrict__ out, int *__restrict__ status) {
    __shared__ double sh_g[kWarpsPerBlock][8][8][3];
    __shared__ double sh_w[kWarpsPerBlock][8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    for (int64_t item = (int64_t)blockIdx.x * kWarpsPerBlock + w; item < n_items;
         item += (int64_t)gridDim.x * kWarpsPerBlock) {
        const int64_t e = elem_list ? elem_list[item] : first + item;
        const int32_t *en = conn + e * 8;
        double xv = 0.0;
        if (lane < 24) xv = coords[(int64_t)en[lane / 3] * 3 + lane % 3];
        // Jacobian at q = lane & 7 (FEBase::init -> libMesh reinit, fe_base.cpp:63-130)
        const int q = lane & 7;
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int a = 0; a < 8; a++) {
            double d[3];
            hex8_dref(q, a, d);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double x = __shfl_sync(full, xv, a * 3 + j);
#pragma unroll
                for (int i = 0; i < 3; i++) J[i * 3 + j] = fma(d[i], x, J[i * 3 + j]);
            }
        }
        double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
        if (lane < 8 && !(det > 0.0)) atomicOr(status, 1);
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
        if (lane < 8) sh_w[w][q] = det;  // unit Gauss weights
        // physical gradients for (q, a) = (p>>3, p&7), p = lane, lane + 32
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int p = lane + 32 * h, qq = p >> 3, a = p & 7;
            double iv[9];
#pragma unroll
            for (int k = 0; k < 9; k++) iv[k] = __shfl_sync(full, inv[k], qq);
            double d[3];
            hex8_dref(qq, a, d);
#pragma unroll
            for (int j = 0; j < 3; j++)
                sh_g[w][qq][a][j] = iv[j * 3] * d[0] + iv[j * 3 + 1] * d[1] + iv[j * 3 + 2] * d[2];
        }
        __syncwarp();
        double acc_mode2 = 0.0;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int p = lane + 32 * h, a = p >> 3, b = p & 7;
            double S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int qq = 0; qq < 8; qq++) {
                // a nodal density field gives the modulus per Gauss point (E_qp), else per element
                const double wq = E_qp ? sh_w[w][qq] * E_qp[e * 8 + qq] : sh_w[w][qq];
                double ga[3], gb[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    ga[i] = wq * sh_g[w][qq][a][i];
                    gb[i] = sh_g[w][qq][b][i];
                }
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) S[i * 3 + j] = fma(ga[i], gb[j], S[i * 3 + j]);
            }
            const double Ee = (MODE == 2 || E_qp) ? 1.0 : E_elem[e];
            const double lam = Ee * lam1, mu = Ee * mu1, tr = S[0] + S[4] + S[8];
            double K[9];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++)
                    K[i * 3 + j] = lam * S[i * 3 + j] + mu * S[j * 3 + i] + (i == j ? mu * tr : 0.0);
            if (MODE == 0) {
                const int64_t na = en[a];
                const int off = emap[e * 64 + a * 8 + b];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    double *dst = vals + rowptr[na * 3 + i] + off;
#pragma unroll
                    for (int j = 0; j < 3; j++) dst[j] += K[i * 3 + j];
                }
            } else if (MODE == 1) {
                double *dst = Ke_out + (e - first) * 576;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) dst[(i * 8 + a) * 24 + j * 8 + b] = K[i * 3 + j];
            } else {
                const int64_t na = en[a], nb = en[b];
                double ua[3], ub[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    ua[i] = (fixed && fixed[na * 3 + i]) ? 0.0 : va[na * 3 + i];
                    ub[i] = (fixed && fixed[nb * 3 + i]) ? 0.0 : vb[nb * 3 + i];
                }
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) acc_mode2 = fma(ua[i] * K[i * 3 + j], ub[j], acc_mode2);
            }
        }
        if (MODE == 2) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc_mode2 += __shfl_xor_sync(full, acc_mode2, o);
            if (lane == 0) out[e] = E_elem[e] * acc_mode2;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Green-Lagrange HEX8 (the NONLINEAR_STRAIN branch, hex8_gl.cuh): one warp per
// element, four warps per block, the element workspace in shared memory.
// MODE 0: scatter the tangent (vals != null) and the internal force (R != null)
// of coloured elements; MODE 1: element tangent (var-blocked) and force;
// MODE 2: out[e] = E_elem[e] a_e . f1_e(X) with f1 the internal force at unit
// modulus (f_int is linear in E at fixed displacement: the density term of the
// adjoint sensitivity, E_elem = dE/drho).
// ---------------------------------------------------------------------------
constexpr int kGlWarps = 4;

template <int MODE>
__global__ void __launch_bounds__(kGlWarps * 32) hex8_gl_kernel(
    const double *__restrict__ coords, const int32_t *__restrict__ conn,
    const int32_t *__restrict__ elem_list, int64_t first, int64_t n_items,
    const double *__restrict__ E_elem, double lam1, double mu1, const double *__restrict__ Xg,
    const int32_t *__restrict__ rowptr, const uint16_t *__restrict__ emap,
    double *__restrict__ vals, double *__restrict__ R, double *__restrict__ Ke_out,
    double *__restrict__ fe_out, const double *__restrict__ va, const uint8_t *__restrict__ fixed,
    double *__restrict__ out, int *__restrict__ status) {
    __shared__ gl::Work sh[kGlWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    gl::Work &s = sh[w];
    for (int64_t item = (int64_t)blockIdx.x * kGlWarps + w; item < n_items;
         item += (int64_t)gridDim.x * kGlWarps) {
        const int64_t e = elem_list ? elem_list[item] : first + item;
        const int32_t *en = conn + e * 8;
        if (lane < 24) {
            const int64_t g = (int64_t)en[lane / 3] * 3 + lane % 3;
            s.X[lane] = coords[g];
            s.u[lane] = Xg[g];
        }
        __syncwarp();
        if (!gl::phase_jacobian(s, lane)) atomicOr(status, 1);
        __syncwarp();
        gl::phase_gradients(s, lane);
        __syncwarp();
        const double Ee = (MODE == 2) ? 1.0 : E_elem[e];
        const double lam = Ee * lam1, mu = Ee * mu1;
        gl::phase_stress(s, lane, lam, mu);
        __syncwarp();
        gl::phase_projections(s, lane);
        __syncwarp();
        if (MODE == 2) {
            double acc = 0.0;
            if (lane < 24) {
                const int64_t g = (int64_t)en[lane / 3] * 3 + lane % 3;
                const double a = (fixed && fixed[g]) ? 0.0 : va[g];
                acc = a * gl::phase_force(s, lane);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) out[e] = E_elem[e] * acc;
        } else {
            if (lane < 24) {
                const int a = lane / 3, i = lane % 3;
                const double fl = gl::phase_force(s, lane);
                if (MODE == 0 && R) R[(int64_t)en[a] * 3 + i] += fl;
                if (MODE == 1 && fe_out) fe_out[(e - first) * 24 + i * 8 + a] = fl;
            }
            if (MODE == 1 || vals) {
#pragma unroll 1
                for (int h = 0; h < 2; h++) {
                    const int p = lane + 32 * h, a = p >> 3, b = p & 7;
                    double K[9];
                    gl::phase_tangent(s, a, b, lam, mu, K);
                    if (MODE == 0) {
                        const int64_t na = en[a];
                        const int off = emap[e * 64 + a * 8 + b];
#pragma unroll
                        for (int i = 0; i < 3; i++) {
                            double *dst = vals + rowptr[na * 3 + i] + off;
#pragma unroll
                            for (int j = 0; j < 3; j++) dst[j] += K[i * 3 + j];
                        }
                    } else {
                        double *dst = Ke_out + (e - first) * 576;
#pragma unroll
                        for (int i = 0; i < 3; i++)
#pragma unroll
                            for (int j = 0; j < 3; j++) dst[(i * 8 + a) * 24 + j * 8 + b] = K[i * 3 + j];
                    }
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// KS stress output (hex8_gl.cuh stress phases): one warp per element, four
// warps per block.  MODE 0: per-element sums over the Gauss points, written
// as four planes of n_el: I_e = sum ex JxW, V_e = sum JxW, A_e = sum vm ex
// JxW, M_e = max vm.  MODE 1 (one colour, atomic-free): g_ia += scale *
// sum_qp ex JxW d vm / d u_ia.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kGlWarps * 32) hex8_stress_kernel(
    const double *__restrict__ coords, const int32_t *__restrict__ conn,
    const int32_t *__restrict__ elem_list, int64_t n_items, const double *__restrict__ Es,
    double lam1, double mu1, int nonlinear, double p_ks, double sigma0,
    const double *__restrict__ Xg, double *__restrict__ sums, int64_t n_el, double scale,
    double *__restrict__ g, int *__restrict__ status) {
    __shared__ gl::StressWork sh[kGlWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    gl::StressWork &s = sh[w];
    for (int64_t item = (int64_t)blockIdx.x * kGlWarps + w; item < n_items;
         item += (int64_t)gridDim.x * kGlWarps) {
        const int64_t e = elem_list ? elem_list[item] : item;
        const int32_t *en = conn + e * 8;
        if (lane < 24) {
            const int64_t gi = (int64_t)en[lane / 3] * 3 + lane % 3;
            s.X[lane] = coords[gi];
            s.u[lane] = Xg[gi];
        }
        __syncwarp();
        if (!gl::phase_jacobian(s, lane)) atomicOr(status, 1);
        __syncwarp();
        gl::phase_gradients(s, lane);
        __syncwarp();
        const double Ee = Es[e];
        gl::phase_von_mises(s, lane, Ee * lam1, Ee * mu1, nonlinear != 0, p_ks, sigma0);
        __syncwarp();
        if (MODE == 0) {
            if (lane == 0) {
                double I = 0.0, V = 0.0, A = 0.0, M = 0.0;
                for (int q = 0; q < 8; q++) {
                    I += s.ex[q] * s.w[q];
                    V += s.w[q];
                    A += s.vm[q] * s.ex[q] * s.w[q];
                    M = fmax(M, s.vm[q]);
                }
                sums[e] = I;
                sums[n_el + e] = V;
                sums[2 * n_el + e] = A;
                sums[3 * n_el + e] = M;
            }
        } else if (lane < 24) {
            g[(int64_t)en[lane / 3] * 3 + lane % 3] += scale * gl::phase_vm_gradient(s, lane);
        }
        __syncwarp();
    }
}

// one block: out = {sum I_e, sum V_e, max M_e} in a fixed order (deterministic)
constexpr int kKsReduceThreads = 1024;
__global__ void __launch_bounds__(kKsReduceThreads) ks_reduce_kernel(const double *__restrict__ sums,
                                                                      int64_t n_el,
                                                                      double *__restrict__ out) {
    __shared__ double sI[kKsReduceThreads], sV[kKsReduceThreads], sM[kKsReduceThreads];
    const int t = threadIdx.x;
    double I = 0.0, V = 0.0, M = 0.0;
    for (int64_t i = t; i < n_el; i += kKsReduceThreads) {
        I += sums[i];
        V += sums[n_el + i];
        M = fmax(M, sums[3 * n_el + i]);
    }
    sI[t] = I;
    sV[t] = V;
    sM[t] = M;
    __syncthreads();
    for (int h = kKsReduceThreads / 2; h > 0; h >>= 1) {
        if (t < h) {
            sI[t] += sI[t + h];
            sV[t] += sV[t + h];
            sM[t] = fmax(sM[t], sM[t + h]);
        }
        __syncthreads();
    }
    if (t == 0) {
        out[0] = sI[0];
        out[1] = sV[0];
        out[2] = sM[0];
    }
}

// out_e = dEs_e / Es_e * A_e * inv_s0I (the direct term through the stress modulus)
//         + adj_e (lambda . dR/drho_e, nullable)
__global__ void ks_combine_kernel(const double *__restrict__ sums, int64_t n_el,
                                  const double *__restrict__ Es, const double *__restrict__ dEs,
                                  double inv_s0I, const double *adj, double *out) {  // adj may be out
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    out[e] = dEs[e] / Es[e] * sums[2 * n_el + e] * inv_s0I + (adj ? adj[e] : 0.0);
}

// Side loads of the elements of one colour (thread per element; elements of a colour
// share no node, so the scatter is atomic-free): HEX8 pressure adds +int phi p n to F,
// QUAD4 heat flux adds -int phi q_n th (the flux enters the residual with +).
__global__ void side_load_kernel(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                 const int32_t *__restrict__ elem_list, int64_t n_items, int hex,
                                 const double *__restrict__ side_vals, double th, double *__restrict__ F) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_items) return;
    const int64_t e = elem_list[t];
    if (hex) {
        const int32_t *en = conn + e * 8;
        double X[24], f[24];
        bool any = false;
        for (int sd = 0; sd < 6; sd++) {
            const double v = side_vals[e * 6 + sd];
            if (v == 0.0) continue;
            if (!any) {
                for (int i = 0; i < 24; i++) {
                    X[i] = coords[(int64_t)en[i / 3] * 3 + i % 3];
                    f[i] = 0.0;
                }
                any = true;
            }
            sl::hex8_pressure_load(X, sd, v, f);
        }
        if (any)
            for (int i = 0; i < 24; i++) F[(int64_t)en[i / 3] * 3 + i % 3] += f[i];
    } else {
        const int32_t *en = conn + e * 4;
        double X[8], f[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < 8; i++) X[i] = coords[(int64_t)en[i / 2] * 2 + i % 2];
        bool any = false;
        for (int sd = 0; sd < 4; sd++) {
            const double v = side_vals[e * 4 + sd];
            if (v == 0.0) continue;
            any = true;
            sl::quad4_flux_load(X, sd, v, th, f);
        }
        if (any)
            for (int a = 0; a < 4; a++) F[en[a]] -= f[a];
    }
}

// y += a x over n entries
__global__ void axpy_kernel(int64_t n, double a, const double *__restrict__ x, double *__restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fma(a, x[i], y[i]);
}

__global__ void zero_fixed_kernel(double *__restrict__ v, const uint8_t *__restrict__ fixed, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && fixed[i]) v[i] = 0.0;
}

// f_e = K_e u_e for element-matrix requests (var-blocked order)
__global__ void elem_matvec_kernel(const double *__restrict__ Ke, const double *__restrict__ X,
                                   const int32_t *__restrict__ conn, int64_t first, int64_t count,
                                   int npe, int dpn, double *__restrict__ fe) {
    const int nd = npe * dpn;
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * nd) return;
    int64_t le = t / nd;
    int row = (int)(t % nd);
    const int32_t *en = conn + (first + le) * npe;
    const double *K = Ke + le * nd * nd + (int64_t)row * nd;
    double s = 0.0;
    for (int c = 0; c < nd; c++) {
        int var = c / npe, node = c % npe;
        s = fma(K[c], X[(int64_t)en[node] * dpn + var], s);
    }
    fe[le * nd + row] = s;
}

// ---------------------------------------------------------------------------
// QUAD4 membrane (StructuralElement2D, linear, NO_BENDING:
// src/elasticity/structural_element_2d.cpp:1076-1227, 1766-1890), thread per
// element.  A = plane-stress C h (isotropic_material_property_card.cpp:395-426).
// MODE 0 scatter, MODE 1 element matrix (8x8 var-blocked).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void membrane_kernel(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                const int32_t *__restrict__ elem_list, int64_t first,
                                int64_t n_items, const double *__restrict__ E_elem, double lam1,
                                double mu1, double h, const int32_t *__restrict__ rowptr,
                                const uint16_t *__restrict__ emap, double *__restrict__ vals,
                                double *__restrict__ Ke_out, int *__restrict__ status) {
    int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items) return;
    const int64_t e = elem_list ? elem_list[item] : first + item;
    const int32_t *en = conn + e * 4;
    double X[8];
    for (int a = 0; a < 4; a++) {
        X[a * 2] = coords[(int64_t)en[a] * 2];
        X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
    }
    double S[4][4][4];
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++)
            for (int k = 0; k < 4; k++) S[a][b][k] = 0.0;
    for (int q = 0; q < 4; q++) {
        double phi[4], g[8];
        double det = quad4_qp(X, q, phi, g);
        if (!(det > 0.0)) atomicOr(status, 1);
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        S[a][b][i * 2 + j] = fma(det * g[a * 2 + i], g[b * 2 + j], S[a][b][i * 2 + j]);
    }
    const double Eh = E_elem[e] * h, lam = Eh * lam1, mu = Eh * mu1;
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) {
            double tr = S[a][b][0] + S[a][b][3];
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++) {
                    double K = lam * S[a][b][i * 2 + j] + mu * S[a][b][j * 2 + i] + (i == j ? mu * tr : 0.0);
                    if (MODE == 0)
                        vals[rowptr[(int64_t)en[a] * 2 + i] + emap[e * 16 + a * 4 + b] + j] += K;
                    else
                        Ke_out[(e - first) * 64 + (i * 4 + a) * 8 + j * 4 + b] = K;
                }
        }
}

// ---------------------------------------------------------------------------
// QUAD4 conduction (HeatConductionElementBase, heat_conduction_elem_base.cpp:
// 53-149 internal, 1100-1154 convection, 1710-1745 source), thread per element.
// k(T) = k0 (1 + beta T_qp) s_e h; consistent adds JxW dT/dx_j dk/dT dB_i^T B.
// MODE 0: scatter R (and K if vals != null); MODE 1: element K and f.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void heat_kernel(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                            const int32_t *__restrict__ elem_list, int64_t first, int64_t n_items,
                            const double *__restrict__ T, double k0, double beta,
                            const double *__restrict__ s_elem, double h,
                            const double *__restrict__ q_elem,
                            const uint8_t *__restrict__ conv_mask, double hc, double Tinf,
                            int consistent, const int32_t *__restrict__ rowptr,
                            const uint16_t *__restrict__ emap, double *__restrict__ vals,
                            double *__restrict__ R, double *__restrict__ Ke_out,
                            double *__restrict__ fe_out, int *__restrict__ status) {
    int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items) return;
    const int64_t e = elem_list ? elem_list[item] : first + item;
    const int32_t *en = conn + e * 4;
    double X[8], Te[4], f[4] = {0, 0, 0, 0}, K[16];
    for (int a = 0; a < 4; a++) {
        X[a * 2] = coords[(int64_t)en[a] * 2];
        X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
        Te[a] = T[en[a]];
    }
    for (int k = 0; k < 16; k++) K[k] = 0.0;
    const double se = s_elem ? s_elem[e] : 1.0;
    const double qe = q_elem ? q_elem[e] : 0.0;
    for (int q = 0; q < 4; q++) {
        double phi[4], g[8];
        double JxW = quad4_qp(X, q, phi, g);
        if (!(JxW > 0.0)) atomicOr(status, 1);
        double Tq = 0, g0 = 0, g1 = 0;
        for (int a = 0; a < 4; a++) {
            Tq = fma(phi[a], Te[a], Tq);
            g0 = fma(g[a * 2], Te[a], g0);
            g1 = fma(g[a * 2 + 1], Te[a], g1);
        }
        const double kq = k0 * (1.0 + beta * Tq) * se * h;
        const double dk = k0 * beta * se * h;
        for (int a = 0; a < 4; a++) {
            f[a] += JxW * (g[a * 2] * kq * g0 + g[a * 2 + 1] * kq * g1);
            f[a] -= JxW * phi[a] * qe * h;  // volume source (th = h)
            for (int b = 0; b < 4; b++) {
                double v = kq * (g[a * 2] * g[b * 2] + g[a * 2 + 1] * g[b * 2 + 1]);
                if (consistent) v += (g[a * 2] * g0 + g[a * 2 + 1] * g1) * dk * phi[b];
                K[a * 4 + b] += JxW * v;
            }
        }
    }
    const uint8_t cm = conv_mask ? conv_mask[e] : 0;
    if (cm) {
        const int sides[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
        for (int s = 0; s < 4; s++) {
            if (!(cm >> s & 1)) continue;
            int n0 = sides[s][0], n1 = sides[s][1];
            double dx = X[n1 * 2] - X[n0 * 2], dy = X[n1 * 2 + 1] - X[n0 * 2 + 1];
            double L = sqrt(dx * dx + dy * dy);
            for (int q = 0; q < 2; q++) {
                double t = gauss_coord(q);
                double JxW = 0.5 * L;
                double phi[4] = {0, 0, 0, 0};
                phi[n0] = 0.5 * (1.0 - t);
                phi[n1] = 0.5 * (1.0 + t);
                double Tq = phi[n0] * Te[n0] + phi[n1] * Te[n1];
                for (int a = 0; a < 4; a++) {
                    f[a] += JxW * phi[a] * h * hc * (Tq - Tinf);
                    for (int b = 0; b < 4; b++) K[a * 4 + b] += JxW * phi[a] * phi[b] * h * hc;
                }
            }
        }
    }
    if (MODE == 0) {
        for (int a = 0; a < 4; a++) {
            if (R) R[en[a]] += f[a];
            if (vals) {
                const int32_t rp = rowptr[en[a]];
                for (int b = 0; b < 4; b++) vals[rp + emap[e * 16 + a * 4 + b]] += K[a * 4 + b];
            }
        }
    } else {
        for (int k = 0; k < 16; k++) Ke_out[(e - first) * 16 + k] = K[k];
        for (int a = 0; a < 4; a++) fe_out[(e - first) * 4 + a] = f[a];
    }
}

// heat parameter sensitivity (internal_residual_sensitivity,
// heat_conduction_elem_base.cpp:553-617): dk/dp = (pa + pb T_qp) h per element.
// kind 0: pa = s_e, pb = s_e beta (k0); kind 1: pa = k0, pb = k0 beta (s_e).
// out_elem[e] = lambda_e . dR_e/dp   (lambda == nullptr: scatter dR/dp into dRdp)
__global__ void heat_sens_kernel(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                 const int32_t *__restrict__ elem_list, int64_t first,
                                 int64_t n_items, const double *__restrict__ T, double k0,
                                 double beta, const double *__restrict__ s_elem, double h, int kind,
                                 const double *__restrict__ lambda, const uint8_t *__restrict__ fixed,
                                 double *__restrict__ out_elem, double *__restrict__ dRdp) {
    int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items) return;
    const int64_t e = elem_list ? elem_list[item] : first + item;
    const int32_t *en = conn + e * 4;
    double X[8], Te[4], df[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; a++) {
        X[a * 2] = coords[(int64_t)en[a] * 2];
        X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
        Te[a] = T[en[a]];
    }
    const double se = s_elem ? s_elem[e] : 1.0;
    const double pa = kind == 0 ? se : k0, pb = kind == 0 ? se * beta : k0 * beta;
    for (int q = 0; q < 4; q++) {
        double phi[4], g[8];
        double JxW = quad4_qp(X, q, phi, g);
        double Tq = 0, g0 = 0, g1 = 0;
        for (int a = 0; a < 4; a++) {
            Tq = fma(phi[a], Te[a], Tq);
            g0 = fma(g[a * 2], Te[a], g0);
            g1 = fma(g[a * 2 + 1], Te[a], g1);
        }
        const double dk = (pa + pb * Tq) * h;
        for (int a = 0; a < 4; a++) df[a] += JxW * dk * (g[a * 2] * g0 + g[a * 2 + 1] * g1);
    }
    if (lambda) {
        double s = 0.0;
        for (int a = 0; a < 4; a++) s = fma(lambda[en[a]], df[a], s);
        out_elem[e] = s;
    } else {
        for (int a = 0; a < 4; a++)
            if (!(fixed && fixed[en[a]])) dRdp[en[a]] += df[a];
    }
}

// lumped weights m_i = sum_e sum_qp JxW phi_i (mean-temperature output)
__global__ void quad4_mass_kernel(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                  const int32_t *__restrict__ elem_list, int64_t n_items,
                                  double *__restrict__ m) {
    int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items) return;
    const int64_t e = elem_list[item];
    const int32_t *en = conn + e * 4;
    double X[8], w[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; a++) {
        X[a * 2] = coords[(int64_t)en[a] * 2];
        X[a * 2 + 1] = coords[(int64_t)en[a] * 2 + 1];
    }
    for (int q = 0; q < 4; q++) {
        double phi[4], g[8];
        double JxW = quad4_qp(X, q, phi, g);
        for (int a = 0; a < 4; a++) w[a] += JxW * phi[a];
    }
    for (int a = 0; a < 4; a++) m[en[a]] += w[a];
}

// element -> CSR column-block offsets (binary search in sorted rows)
__global__ void emap_kernel(const int32_t *__restrict__ conn, int64_t n_elems, int npe, int dpn,
                            const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                            uint16_t *__restrict__ emap, int *__restrict__ status) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t pairs = (int64_t)npe * npe;
    if (t >= n_elems * pairs) return;
    int64_t e = t / pairs;
    int ab = (int)(t % pairs), a = ab / npe, b = ab % npe;
    int64_t row = (int64_t)conn[e * npe + a] * dpn;
    int32_t target = conn[e * npe + b] * dpn;
    int32_t lo = rowptr[row], hi = rowptr[row + 1] - 1, pos = -1;
    while (lo <= hi) {
        int32_t mid = (lo + hi) >> 1, c = cols[mid];
        if (c == target) { pos = mid; break; }
        if (c < target) lo = mid + 1; else hi = mid - 1;
    }
    if (pos < 0 || pos - rowptr[row] > 65535) {
        atomicOr(status, 2);
        emap[t] = 0;
    } else {
        emap[t] = (uint16_t)(pos - rowptr[row]);
    }
}

__global__ void fix_kernel(double *__restrict__ vals, const int64_t *__restrict__ zero_pos,
                           int64_t n_zero, const int64_t *__restrict__ diag_pos, int64_t n_diag) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n_zero) vals[zero_pos[t]] = 0.0;
    if (t < n_diag) vals[diag_pos[t]] = 1.0;
}

// SIMP modulus (examples/structural/example_6/example_6.cpp:100-137)
__global__ void simp_modulus_kernel(const double *__restrict__ rho, int64_t n, double E0,
                                    double rmin, double penal, double *__restrict__ E,
                                    double *__restrict__ dE, int *__restrict__ status) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double r = rho ? rho[e] : 1.0;
    if (!(r >= 0.0 && r <= 1.0)) atomicOr(status, 4);  // NaN or out of range
    double rp, rp1;
    const int ip = (int)penal;
    if ((double)ip == penal && ip >= 1 && ip <= 8) {
        // integer penalty: repeated products (FP64 pow is slow on this part)
        rp1 = 1.0;
        for (int k = 1; k < ip; k++) rp1 *= r;
        rp = rp1 * r;
    } else {
        rp = pow(r, penal);
        rp1 = pow(r, penal - 1.0);
    }
    E[e] = E0 * (rmin + (1.0 - rmin) * rp);
    dE[e] = E0 * (1.0 - rmin) * penal * rp1;
}

// SIMP modulus of a nodal density field (the MeshFieldFunction "rho" of
// example_6.cpp:104-137 over FIRST-order LAGRANGE, :250-252): rho at Gauss point
// q of element e is sum_a N_a(x_q) rho_a (the trilinear shape functions, the same
// points as the element kernels), E_q = E0 (rmin + (1 - rmin) rho_q^p), dE_q/drho_q.
// One thread per (element, point); rho_a outside [0, 1] or NaN sets status bit 4.
__global__ void simp_nodal_modulus_kernel(const int32_t *__restrict__ conn, const double *__restrict__ rho,
                                          int64_t n_elems, double E0, double rmin, double penal,
                                          double *__restrict__ Eq, double *__restrict__ dEq,
                                          int *__restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_elems * 8) return;
    const int64_t e = t >> 3;
    const int q = (int)(t & 7);
    const double xi = gauss_coord(q & 1), eta = gauss_coord(q >> 1 & 1), zeta = gauss_coord(q >> 2 & 1);
    double r = 0.0;
#pragma unroll
    for (int a = 0; a < 8; a++) {
        double sx, sy, sz;
        hex8_sign(a, sx, sy, sz);
        const double ra = rho[conn[e * 8 + a]];
        if (!(ra >= 0.0 && ra <= 1.0)) atomicOr(status, 4);
        r = fma(0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta), ra, r);
    }
    double rp, rp1;
    const int ip = (int)penal;
    if ((double)ip == penal && ip >= 1 && ip <= 8) {
        rp1 = 1.0;
        for (int k = 1; k < ip; k++) rp1 *= r;
        rp = rp1 * r;
    } else {
        rp = pow(r, penal);
        rp1 = pow(r, penal - 1.0);
    }
    Eq[t] = E0 * (rmin + (1.0 - rmin) * rp);
    dEq[t] = E0 * (1.0 - rmin) * penal * rp1;
}

// Strain energy at each Gauss point at unit modulus, times dE_q/drho_q:
// out[8 e + q] = dE_q det J_q (lam1 tr(eps)^2 + 2 mu1 eps : eps), eps the linear strain
// of u at point q (unit Gauss weights; constrained dofs read as 0).  One warp per
// element, lanes 0-7 one point each.
__global__ void __launch_bounds__(256) hex8_qp_energy_kernel(
    const double *__restrict__ coords, const int32_t *__restrict__ conn, int64_t n_elems,
    const double *__restrict__ dEq, double lam1, double mu1, const double *__restrict__ u,
    const uint8_t *__restrict__ fixed, double *__restrict__ out) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    for (int64_t e = (int64_t)blockIdx.x * kWarpsPerBlock + w; e < n_elems; e += (int64_t)gridDim.x * kWarpsPerBlock) {
        const int32_t *en = conn + e * 8;
        double xv = 0.0, uv = 0.0;
        if (lane < 24) {
            const int64_t g = (int64_t)en[lane / 3] * 3 + lane % 3;
            xv = coords[g];
            uv = (fixed && fixed[g]) ? 0.0 : u[g];
        }
        const int q = lane & 7;
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int a = 0; a < 8; a++) {
            double d[3];
            hex8_dref(q, a, d);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const double x = __shfl_sync(full, xv, a * 3 + j);
#pragma unroll
                for (int i = 0; i < 3; i++) J[i * 3 + j] = fma(d[i], x, J[i * 3 + j]);
            }
        }
        const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
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
        double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // H[i][j] = d u_i / d x_j
#pragma unroll
        for (int a = 0; a < 8; a++) {
            double d[3];
            hex8_dref(q, a, d);
            double g[3];
#pragma unroll
            for (int j = 0; j < 3; j++) g[j] = inv[j * 3] * d[0] + inv[j * 3 + 1] * d[1] + inv[j * 3 + 2] * d[2];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const double ua = __shfl_sync(full, uv, a * 3 + i);
#pragma unroll
                for (int j = 0; j < 3; j++) H[i * 3 + j] = fma(ua, g[j], H[i * 3 + j]);
            }
        }
        const double tr = H[0] + H[4] + H[8];
        double ee = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const double eij = 0.5 * (H[i * 3 + j] + H[j * 3 + i]);
                ee = fma(eij, eij, ee);
            }
        if (lane < 8) out[e * 8 + q] = dEq[e * 8 + q] * det * (lam1 * tr * tr + 2.0 * mu1 * ee);
    }
}

// dc[n] = -sum over the (element, corner) incidences of node n, in element order,
// of sum_q N_corner(x_q) out[8 e + q]
__global__ void nodal_gather_kernel(const int32_t *__restrict__ ptr, const int32_t *__restrict__ inc,
                                    int64_t n_nodes, const double *__restrict__ out,
                                    double *__restrict__ dc) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= n_nodes) return;
    double s = 0.0;
    for (int32_t k = ptr[n]; k < ptr[n + 1]; k++) {
        const int64_t e = inc[k] >> 3;
        const int a = inc[k] & 7;
        double sx, sy, sz;
        hex8_sign(a, sx, sy, sz);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const double xi = gauss_coord(q & 1), eta = gauss_coord(q >> 1 & 1), zeta = gauss_coord(q >> 2 & 1);
            s = fma(0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta), out[e * 8 + q], s);
        }
    }
    dc[n] = -s;
}

// residual fix-up: constrained rows R_d = X_d, point loads enter as -F
__global__ void residual_finish_kernel(double *__restrict__ R, const double *__restrict__ X,
                                       const double *__restrict__ F, const uint8_t *__restrict__ fixed,
                                       int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r = R[i] - (F ? F[i] : 0.0);
    if (fixed && fixed[i]) r = X[i];
    R[i] = r;
}

int read_status(mg_problem *p, int *d_status) {
    int h = 0;
    MG_CUDA_TRY(cudaMemcpyAsync(&h, d_status, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    if (h & 1) { set_error("element with non-positive Jacobian determinant"); return MG_EBADELEM; }
    if (h & 2) { set_error("element/CSR map inconsistent with the sparsity pattern"); return MG_EINVAL; }
    if (h & 4) { set_error("design density outside [0,1] or NaN"); return MG_EINVAL; }
    return MG_OK;
}

int *status_slot(mg_problem *p) {
    // last int of the reduction scratch is the kernel status word
    return reinterpret_cast<int *>(p->d_red + 2 * p->red_blocks + 6);
}

inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void lame_3d(double nu, double &lam1, double &mu1) {
    lam1 = nu / (1.0 - nu - 2.0 * nu * nu);
    mu1 = 1.0 / (2.0 * (1.0 + nu));
}

}  // namespace

int compute_modulus(mg_problem *p) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    double rmin = p->mat.Emin / p->mat.E0;
    simp_modulus_kernel<<<blocks_for(p->n_elems, 256), 256, 0, p->stream>>>(
        p->d_rho, p->n_elems, p->mat.E0, rmin, p->mat.penal, p->d_E, p->d_dE, st);
    MG_CUDA_TRY(cudaGetLastError());
    return read_status(p, st);
}

int compute_nodal_modulus(mg_problem *p) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    const double rmin = p->mat.Emin / p->mat.E0;
    simp_nodal_modulus_kernel<<<blocks_for(p->n_elems * 8, 256), 256, 0, p->stream>>>(
        p->d_conn, p->d_rho_nodes, p->n_elems, p->mat.E0, rmin, p->mat.penal, p->d_Eq, p->d_dEq, st);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return read_status(p, st);
}

// dC/drho_n of the compliance C = F.u at the solution u (the adjoint is -u):
// -u^T dK/drho_n u, dK/drho_n = sum over the node's elements and Gauss points of
// dE_q N_n(x_q) K1_q (K1_q the unit-modulus stiffness of point q); n_nodes values
// into dc_dev
int nodal_compliance_sensitivity(mg_problem *p, const double *d_u, double *dc_dev) {
    double lam1, mu1;
    lame_3d(p->mat.nu, lam1, mu1);
    hex8_qp_energy_kernel<<<std::max(1u, std::min(blocks_for(p->n_elems, kWarpsPerBlock), 65535u)), 256, 0,
                            p->stream>>>(p->d_coords, p->d_conn, p->n_elems, p->d_dEq, lam1, mu1, d_u,
                                         p->d_fixed, p->d_qp_out);
    MG_CUDA_TRY(cudaGetLastError());
    nodal_gather_kernel<<<blocks_for(p->n_nodes, 256), 256, 0, p->stream>>>(
        p->d_node_inc_ptr, p->d_node_inc, p->n_nodes, p->d_qp_out, dc_dev);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(2);
    return MG_OK;
}

int launch_simp_modulus(const double *d_rho, int64_t n, const mg_material_desc &mat, double *d_E,
                        double *d_dE, int *d_status, cudaStream_t s) {
    if (n <= 0) return MG_OK;
    simp_modulus_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d_rho, n, mat.E0, mat.Emin / mat.E0,
                                                           mat.penal, d_E, d_dE, d_status);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return MG_OK;
}

int build_emap(mg_problem *p) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    int64_t total = p->n_elems * p->npe * p->npe;
    emap_kernel<<<blocks_for(total, 256), 256, 0, p->stream>>>(
        p->d_conn, p->n_elems, p->npe, p->dpn, p->A.rowptr, p->A.cols, p->d_emap, st);
    MG_CUDA_TRY(cudaGetLastError());
    return read_status(p, st);
}

int assemble_system(mg_problem *p, const double *d_X, double *d_R, bool want_jacobian,
                    bool consistent) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    const bool need_K = want_jacobian || (p->physics != MG_PHYSICS_HEAT_QUAD4 && d_R);
    if (p->physics == MG_PHYSICS_HEAT_QUAD4) {
        if (want_jacobian)
            MG_CUDA_TRY(cudaMemsetAsync(p->A.vals, 0, p->A.nnz * sizeof(double), p->stream));
        if (d_R) MG_CUDA_TRY(cudaMemsetAsync(d_R, 0, p->n_dofs * sizeof(double), p->stream));
        for (int c = 0; c < p->n_colors; c++) {
            int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
            heat_kernel<0><<<blocks_for(cnt, 128), 128, 0, p->stream>>>(
                p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, d_X,
                p->mat.k0, p->mat.k_beta, p->d_s, p->mat.thickness, p->d_q, p->d_conv_mask,
                p->conv_h, p->conv_Tinf, consistent ? 1 : 0, p->A.rowptr, p->d_emap,
                want_jacobian ? p->A.vals : nullptr, d_R, nullptr, nullptr, st);
            MG_CUDA_TRY(cudaGetLastError());
        }
        if (want_jacobian && (p->n_fix_zero || p->n_fix_diag)) {
            int64_t m = p->n_fix_zero > p->n_fix_diag ? p->n_fix_zero : p->n_fix_diag;
            fix_kernel<<<blocks_for(m, 256), 256, 0, p->stream>>>(p->A.vals, p->d_fix_zero,
                                                                  p->n_fix_zero, p->d_fix_diag,
                                                                  p->n_fix_diag);
            MG_CUDA_TRY(cudaGetLastError());
        }
        if (d_R) {
            residual_finish_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(
                d_R, d_X, p->d_F, p->d_fixed, p->n_dofs);
            MG_CUDA_TRY(cudaGetLastError());
        }
        MG_TRY(read_status(p, st));
        if (want_jacobian) p->jacobian_valid = true;
        return MG_OK;
    }
    if (p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        // tangent and internal force both depend on X: R = f_int(X) - F
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        if (want_jacobian)
            MG_CUDA_TRY(cudaMemsetAsync(p->A.vals, 0, p->A.nnz * sizeof(double), p->stream));
        if (d_R) MG_CUDA_TRY(cudaMemsetAsync(d_R, 0, p->n_dofs * sizeof(double), p->stream));
        for (int c = 0; c < p->n_colors; c++) {
            int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
            hex8_gl_kernel<0><<<blocks_for(cnt, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
                p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, p->d_E, lam1,
                mu1, d_X, p->A.rowptr, p->d_emap, want_jacobian ? p->A.vals : nullptr, d_R, nullptr,
                nullptr, nullptr, nullptr, nullptr, st);
            MG_CUDA_TRY(cudaGetLastError());
        }
        count_launches(p->n_colors);
        if (want_jacobian && (p->n_fix_zero || p->n_fix_diag)) {
            int64_t m = p->n_fix_zero > p->n_fix_diag ? p->n_fix_zero : p->n_fix_diag;
            fix_kernel<<<blocks_for(m, 256), 256, 0, p->stream>>>(p->A.vals, p->d_fix_zero,
                                                                  p->n_fix_zero, p->d_fix_diag,
                                                                  p->n_fix_diag);
            MG_CUDA_TRY(cudaGetLastError());
        }
        if (d_R) {
            residual_finish_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(
                d_R, d_X, p->d_F, p->d_fixed, p->n_dofs);
            MG_CUDA_TRY(cudaGetLastError());
        }
        MG_TRY(read_status(p, st));
        // the CSR holds the tangent at this X only
        p->jacobian_valid = false;
        return MG_OK;
    }
    // linear elasticity / membrane: K depends on the design only
    if (need_K && !p->jacobian_valid) {
        MG_CUDA_TRY(cudaMemsetAsync(p->A.vals, 0, p->A.nnz * sizeof(double), p->stream));
        double lam1, mu1;
        if (p->physics == MG_PHYSICS_ELASTICITY_HEX8) {
            lame_3d(p->mat.nu, lam1, mu1);
            for (int c = 0; c < p->n_colors; c++) {
                int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
                unsigned grid = blocks_for(cnt, kWarpsPerBlock);
                hex8_kernel<0><<<grid, 256, 0, p->stream>>>(
                    p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, p->d_E,
                    p->nodal_design ? p->d_Eq : nullptr, lam1, mu1, p->A.rowptr, p->d_emap, p->A.vals,
                    nullptr, nullptr, nullptr, nullptr, nullptr, st);
                MG_CUDA_TRY(cudaGetLastError());
            }
        } else {
            double nu = p->mat.nu;
            lam1 = nu / (1.0 - nu * nu);
            mu1 = 1.0 / (2.0 * (1.0 + nu));
            for (int c = 0; c < p->n_colors; c++) {
                int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
                membrane_kernel<0><<<blocks_for(cnt, 128), 128, 0, p->stream>>>(
                    p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, p->d_E,
                    lam1, mu1, p->mat.thickness, p->A.rowptr, p->d_emap, p->A.vals, nullptr, st);
                MG_CUDA_TRY(cudaGetLastError());
            }
        }
        if (p->n_fix_zero || p->n_fix_diag) {
            int64_t m = p->n_fix_zero > p->n_fix_diag ? p->n_fix_zero : p->n_fix_diag;
            fix_kernel<<<blocks_for(m, 256), 256, 0, p->stream>>>(p->A.vals, p->d_fix_zero,
                                                                  p->n_fix_zero, p->d_fix_diag,
                                                                  p->n_fix_diag);
            MG_CUDA_TRY(cudaGetLastError());
        }
        MG_TRY(read_status(p, st));
        p->jacobian_valid = true;
    }
    if (d_R) {
        // R = K X - F (linear internal force; Dirichlet rows carry R_d = X_d)
        MG_TRY(spmv(p, p->A, d_X, d_R));
        residual_finish_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(
            d_R, d_X, p->d_F, p->d_fixed, p->n_dofs);
        MG_CUDA_TRY(cudaGetLastError());
    }
    return MG_OK;
}

// d_F = the point loads + the side loads of p->d_side (nullable), zero on constrained
// dofs; h_F receives a copy for the host-side consumers (the mixed form's set-up)
int assemble_side_loads(mg_problem *p) {
    MG_CUDA_TRY(cudaMemcpyAsync(p->d_F, p->h_F_point.data(), p->n_dofs * sizeof(double),
                                cudaMemcpyHostToDevice, p->stream));
    if (p->d_side) {
        const int hex = p->dim == 3;
        for (int c = 0; c < p->n_colors; c++) {
            int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
            side_load_kernel<<<blocks_for(cnt, 128), 128, 0, p->stream>>>(
                p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], cnt, hex, p->d_side,
                p->mat.thickness, p->d_F);
            MG_CUDA_TRY(cudaGetLastError());
        }
        count_launches(p->n_colors);
    }
    zero_fixed_kernel<<<blocks_for(p->n_dofs, 256), 256, 0, p->stream>>>(p->d_F, p->d_fixed, p->n_dofs);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    MG_CUDA_TRY(cudaMemcpyAsync(p->h_F.data(), p->d_F, p->n_dofs * sizeof(double), cudaMemcpyDeviceToHost,
                                p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

// KS stress output, value pass: stress modulus Es(rho) at SIMP exponent `penal` into
// ks[0, n_el), dEs into ks[n_el, 2 n_el), the element sums into ks[2 n_el, 6 n_el) and
// {I, V, max vm} into ks[6 n_el, 6 n_el + 3); returns the three scalars on the host
int ks_stress_values(mg_problem *p, const double *d_X, double p_ks, double sigma0, double penal,
                     double *d_ks, double host_out[3]) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    const int64_t n = p->n_elems;
    mg_material_desc ms = p->mat;
    ms.penal = penal;
    MG_TRY(launch_simp_modulus(p->d_rho, n, ms, d_ks, d_ks + n, st, p->stream));
    double lam1, mu1;
    lame_3d(p->mat.nu, lam1, mu1);
    const int nonlinear = p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR;
    hex8_stress_kernel<0><<<blocks_for(n, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
        p->d_coords, p->d_conn, nullptr, n, d_ks, lam1, mu1, nonlinear, p_ks, sigma0, d_X,
        d_ks + 2 * n, n, 0.0, nullptr, st);
    MG_CUDA_TRY(cudaGetLastError());
    ks_reduce_kernel<<<1, kKsReduceThreads, 0, p->stream>>>(d_ks + 2 * n, n, d_ks + 6 * n);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(3);
    MG_CUDA_TRY(cudaMemcpyAsync(host_out, d_ks + 6 * n, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                p->stream));
    return read_status(p, st);  // synchronises
}

// KS stress output, gradient pass: d_g = scale * d(sum_qp ex JxW)/du ... scattered per colour
// (d_g zeroed first); uses the stress modulus left in d_ks by ks_stress_values
int ks_stress_gradient(mg_problem *p, const double *d_X, double p_ks, double sigma0,
                       const double *d_ks, double scale, double *d_g) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    MG_CUDA_TRY(cudaMemsetAsync(d_g, 0, p->n_dofs * sizeof(double), p->stream));
    double lam1, mu1;
    lame_3d(p->mat.nu, lam1, mu1);
    const int nonlinear = p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR;
    for (int c = 0; c < p->n_colors; c++) {
        int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
        hex8_stress_kernel<1><<<blocks_for(cnt, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
            p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], cnt, d_ks, lam1, mu1,
            nonlinear, p_ks, sigma0, d_X, nullptr, p->n_elems, scale, d_g, st);
        MG_CUDA_TRY(cudaGetLastError());
    }
    count_launches(p->n_colors);
    return read_status(p, st);
}

// d_out_e = direct term + d_adj_e (nullable)
int ks_stress_combine(mg_problem *p, const double *d_ks, double inv_s0I, const double *d_adj,
                      double *d_out) {
    const int64_t n = p->n_elems;
    ks_combine_kernel<<<blocks_for(n, 256), 256, 0, p->stream>>>(d_ks + 2 * n, n, d_ks, d_ks + n,
                                                                  inv_s0I, d_adj, d_out);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return MG_OK;
}

// `reps` assemblies of the nonlinear-strain residual and tangent at d_X, enqueued on the
// handle's stream without synchronising (event timing of the element kernel)
int launch_assembly(mg_problem *p, const double *d_X, int reps) {
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        set_error("assembly launch hook: nonlinear-strain HEX8 only");
        return MG_ENOTSUP;
    }
    int *st = status_slot(p);
    double lam1, mu1;
    lame_3d(p->mat.nu, lam1, mu1);
    for (int r = 0; r < reps; r++) {
        MG_CUDA_TRY(cudaMemsetAsync(p->A.vals, 0, p->A.nnz * sizeof(double), p->stream));
        MG_CUDA_TRY(cudaMemsetAsync(p->d_R, 0, p->n_dofs * sizeof(double), p->stream));
        for (int c = 0; c < p->n_colors; c++) {
            int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
            hex8_gl_kernel<0><<<blocks_for(cnt, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
                p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, p->d_E, lam1,
                mu1, d_X, p->A.rowptr, p->d_emap, p->A.vals, p->d_R, nullptr, nullptr, nullptr,
                nullptr, nullptr, st);
            MG_CUDA_TRY(cudaGetLastError());
        }
    }
    count_launches((long long)reps * p->n_colors);
    p->jacobian_valid = false;
    return MG_OK;
}

int element_matrices(mg_problem *p, const double *d_X, int64_t first, int64_t count,
                     double *d_Ke, double *d_fe) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    const int nd = p->npe * p->dpn;
    if (p->physics == MG_PHYSICS_ELASTICITY_HEX8) {
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        hex8_kernel<1><<<blocks_for(count, kWarpsPerBlock), 256, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, first, count, p->d_E, p->nodal_design ? p->d_Eq : nullptr,
            lam1, mu1, nullptr, nullptr, nullptr, d_Ke, nullptr, nullptr, nullptr, nullptr, st);
    } else if (p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        hex8_gl_kernel<1><<<blocks_for(count, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, first, count, p->d_E, lam1, mu1, d_X, nullptr,
            nullptr, nullptr, nullptr, d_Ke, d_fe, nullptr, nullptr, nullptr, st);
    } else if (p->physics == MG_PHYSICS_MEMBRANE_QUAD4) {
        double nu = p->mat.nu;
        membrane_kernel<1><<<blocks_for(count, 128), 128, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, first, count, p->d_E, nu / (1.0 - nu * nu),
            1.0 / (2.0 * (1.0 + nu)), p->mat.thickness, nullptr, nullptr, nullptr, d_Ke, st);
    } else {
        heat_kernel<1><<<blocks_for(count, 128), 128, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, first, count, d_X, p->mat.k0, p->mat.k_beta, p->d_s,
            p->mat.thickness, p->d_q, p->d_conv_mask, p->conv_h, p->conv_Tinf, 1, nullptr,
            nullptr, nullptr, nullptr, d_Ke, d_fe, st);
    }
    MG_CUDA_TRY(cudaGetLastError());
    if (p->physics != MG_PHYSICS_HEAT_QUAD4 && p->physics != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR &&
        d_fe) {
        elem_matvec_kernel<<<blocks_for(count * nd, 128), 128, 0, p->stream>>>(
            d_Ke, d_X, p->d_conn, first, count, p->npe, p->dpn, d_fe);
        MG_CUDA_TRY(cudaGetLastError());
    }
    return read_status(p, st);
}

// Per-element adjoint sensitivity contributions.
//  elasticity, kind MG_PARAM_DENSITY: out[e] = dE_e lambda_e^T K1_e X_e
//  heat, kind MG_PARAM_K0 / MG_PARAM_ELEM_SCALE: out[e] = lambda_e . dR_e/dp
int elem_sensitivity(mg_problem *p, const double *d_X, const double *d_lambda, int kind,
                     double *d_out_elem) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    if (p->physics == MG_PHYSICS_ELASTICITY_HEX8 && kind == MG_PARAM_DENSITY) {
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        hex8_kernel<2><<<blocks_for(p->n_elems, kWarpsPerBlock), 256, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, 0, p->n_elems, p->d_dE, nullptr, lam1, mu1, nullptr,
            nullptr, nullptr, nullptr, d_lambda, d_X, p->d_fixed, d_out_elem, st);
    } else if (p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR && kind == MG_PARAM_DENSITY) {
        // out[e] = dE_e lambda_e . f1_e(X)
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        hex8_gl_kernel<2><<<blocks_for(p->n_elems, kGlWarps), kGlWarps * 32, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, 0, p->n_elems, p->d_dE, lam1, mu1, d_X, nullptr,
            nullptr, nullptr, nullptr, nullptr, nullptr, d_lambda, p->d_fixed, d_out_elem, st);
    } else if (p->physics == MG_PHYSICS_HEAT_QUAD4 &&
               (kind == MG_PARAM_K0 || kind == MG_PARAM_ELEM_SCALE)) {
        heat_sens_kernel<<<blocks_for(p->n_elems, 128), 128, 0, p->stream>>>(
            p->d_coords, p->d_conn, nullptr, 0, p->n_elems, d_X, p->mat.k0, p->mat.k_beta, p->d_s,
            p->mat.thickness, kind == MG_PARAM_K0 ? 0 : 1, d_lambda, p->d_fixed, d_out_elem,
            nullptr);
    } else {
        set_error("sensitivity kind %d not available for this physics", kind);
        return MG_ENOTSUP;
    }
    MG_CUDA_TRY(cudaGetLastError());
    return read_status(p, st);
}

// dR/dp as a global vector (NonlinearImplicitAssembly::sensitivity_assemble,
// nonlinear_implicit_assembly.cpp:515-686); constrained rows are zero.
int assemble_param_residual(mg_problem *p, const double *d_X, int kind, int64_t index,
                            double *d_dRdp) {
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    MG_CUDA_TRY(cudaMemsetAsync(d_dRdp, 0, p->n_dofs * sizeof(double), p->stream));
    if ((p->physics == MG_PHYSICS_ELASTICITY_HEX8 ||
         p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) && kind == MG_PARAM_DENSITY) {
        if (index < 0 || index >= p->n_elems) return MG_EINVAL;
        // one element: f = dE K1 X_e (linear) or dE f1(X_e) (nonlinear strain: f_int is
        // linear in E at fixed X), scattered on the host (single element: no races)
        double *Ke = p->d_tmp2;  // needs 600 doubles
        double *fe = Ke + 576;
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        if (p->physics == MG_PHYSICS_ELASTICITY_HEX8) {
            hex8_kernel<1><<<1, 256, 0, p->stream>>>(p->d_coords, p->d_conn, nullptr, index, 1,
                                                     p->d_dE, nullptr, lam1, mu1, nullptr, nullptr,
                                                     nullptr, Ke, nullptr, nullptr, nullptr, nullptr, st);
            MG_CUDA_TRY(cudaGetLastError());
            elem_matvec_kernel<<<1, 32, 0, p->stream>>>(Ke, d_X, p->d_conn, index, 1, 8, 3, fe);
        } else {
            hex8_gl_kernel<1><<<1, kGlWarps * 32, 0, p->stream>>>(
                p->d_coords, p->d_conn, nullptr, index, 1, p->d_dE, lam1, mu1, d_X, nullptr,
                nullptr, nullptr, nullptr, Ke, fe, nullptr, nullptr, nullptr, st);
        }
        MG_CUDA_TRY(cudaGetLastError());
        std::vector<double> hfe(24);
        std::vector<int32_t> en(8);
        MG_CUDA_TRY(cudaMemcpyAsync(hfe.data(), fe, 24 * sizeof(double), cudaMemcpyDeviceToHost,
                                    p->stream));
        MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
        std::vector<double> hvec(24);
        for (int a = 0; a < 8; a++) en[a] = p->h_conn[index * 8 + a];
        for (int a = 0; a < 8; a++)
            for (int i = 0; i < 3; i++) {
                int64_t g = (int64_t)en[a] * 3 + i;
                double v = p->h_fixed[g] ? 0.0 : hfe[i * 8 + a];
                MG_CUDA_TRY(cudaMemcpyAsync(d_dRdp + g, &v, sizeof(double), cudaMemcpyHostToDevice,
                                            p->stream));
                MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
            }
        return read_status(p, st);
    }
    if (p->physics == MG_PHYSICS_HEAT_QUAD4 && kind == MG_PARAM_K0) {
        for (int c = 0; c < p->n_colors; c++) {
            int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
            heat_sens_kernel<<<blocks_for(cnt, 128), 128, 0, p->stream>>>(
                p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], 0, cnt, d_X,
                p->mat.k0, p->mat.k_beta, p->d_s, p->mat.thickness, 0, nullptr, p->d_fixed,
                nullptr, d_dRdp);
            MG_CUDA_TRY(cudaGetLastError());
        }
        return read_status(p, st);
    }
    if (p->physics == MG_PHYSICS_HEAT_QUAD4 && kind == MG_PARAM_ELEM_SCALE) {
        if (index < 0 || index >= p->n_elems) return MG_EINVAL;
        heat_sens_kernel<<<1, 32, 0, p->stream>>>(p->d_coords, p->d_conn, nullptr, index, 1, d_X,
                                                  p->mat.k0, p->mat.k_beta, p->d_s,
                                                  p->mat.thickness, 1, nullptr, p->d_fixed,
                                                  nullptr, d_dRdp);
        MG_CUDA_TRY(cudaGetLastError());
        return read_status(p, st);
    }
    set_error("parameter kind %d not available for this physics", kind);
    return MG_ENOTSUP;
}

// ---------------------------------------------------------------------------
// Per-element plugin calls (NonlinearImplicitAssemblyElemOperations::elem_calculations
// and elem_sensitivity_calculations, nonlinear_implicit_assembly_elem_operations.h:50-105,
// after init(elem) and set_elem_solution(sol), assembly_elem_operation.h:94-139).  The
// element-local solution (var-blocked: component c of local node a at c * npe + a) is
// scattered into a zeroed global vector; only element e's own dofs are read from it.
__global__ void elem_scatter_kernel(const double *__restrict__ sol, const int32_t *__restrict__ conn,
                                    int64_t e, int npe, int dpn, double *__restrict__ X) {
    const int t = threadIdx.x;
    if (t >= npe * dpn) return;
    const int c = t / npe, a = t - c * npe;
    X[(int64_t)conn[e * npe + a] * dpn + c] = sol[t];
}

__global__ void elem_gather_kernel(const double *__restrict__ X, const int32_t *__restrict__ conn,
                                   int64_t e, int npe, int dpn, double *__restrict__ out) {
    const int t = threadIdx.x;
    if (t >= npe * dpn) return;
    const int c = t / npe, a = t - c * npe;
    out[t] = X[(int64_t)conn[e * npe + a] * dpn + c];
}

// d_sol: the element-local solution (device); d_Ke, d_fe (nullable) receive the element
// Jacobian and the element residual f_int - f_ext of the element's own loads (heat:
// convection and volume source; every physics: its side loads).  Uses d_tmp, d_tmp2.
int element_calculations(mg_problem *p, int64_t e, const double *d_sol, double *d_Ke,
                         double *d_fe, int32_t *d_elem_slot) {
    const int nd = p->npe * p->dpn;
    MG_CUDA_TRY(cudaMemsetAsync(p->d_tmp, 0, p->n_dofs * sizeof(double), p->stream));
    elem_scatter_kernel<<<1, 64, 0, p->stream>>>(d_sol, p->d_conn, e, p->npe, p->dpn, p->d_tmp);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    MG_TRY(element_matrices(p, p->d_tmp, e, 1, d_Ke, d_fe));
    if (d_fe && p->d_side) {
        // the element's side loads: F_e of side_load_kernel on this one element, then
        // f_e -= F_e (the residual convention R = f_int - f_ext)
        const int hex = (p->physics == MG_PHYSICS_ELASTICITY_HEX8 ||
                         p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) ? 1 : 0;
        const int32_t e32 = (int32_t)e;
        MG_CUDA_TRY(cudaMemcpyAsync(d_elem_slot, &e32, sizeof(int32_t), cudaMemcpyHostToDevice, p->stream));
        MG_CUDA_TRY(cudaMemsetAsync(p->d_tmp2, 0, p->n_dofs * sizeof(double), p->stream));
        side_load_kernel<<<1, 32, 0, p->stream>>>(p->d_coords, p->d_conn, d_elem_slot, 1, hex, p->d_side,
                                                  p->mat.thickness, p->d_tmp2);
        MG_CUDA_TRY(cudaGetLastError());
        double *d_Fe = p->d_tmp;  // the scattered solution is no longer needed
        elem_gather_kernel<<<1, 64, 0, p->stream>>>(p->d_tmp2, p->d_conn, e, p->npe, p->dpn, d_Fe);
        MG_CUDA_TRY(cudaGetLastError());
        axpy_kernel<<<1, 64, 0, p->stream>>>(nd, -1.0, d_Fe, d_fe);
        MG_CUDA_TRY(cudaGetLastError());
        count_launches(3);
        MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    }
    return MG_OK;
}

// d/dp of element e's residual at the element-local solution d_sol for the parameter
// (kind, index) of mg_sensitivity_assemble, into d_dfe (device, npe * dpn).  Element
// parameters of other elements give zero.  Uses d_tmp, d_tmp2.
int element_sensitivity(mg_problem *p, int64_t e, const double *d_sol, int kind, int64_t index,
                        double *d_dfe) {
    const int nd = p->npe * p->dpn;
    int *st = status_slot(p);
    MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(int), p->stream));
    MG_CUDA_TRY(cudaMemsetAsync(d_dfe, 0, nd * sizeof(double), p->stream));
    const bool elast = p->physics == MG_PHYSICS_ELASTICITY_HEX8 ||
                       p->physics == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR;
    const bool heat = p->physics == MG_PHYSICS_HEAT_QUAD4;
    if (!((elast && kind == MG_PARAM_DENSITY) ||
          (heat && (kind == MG_PARAM_K0 || kind == MG_PARAM_ELEM_SCALE)))) {
        set_error("parameter kind %d not available for this physics", kind);
        return MG_ENOTSUP;
    }
    if (kind != MG_PARAM_K0 && (index < 0 || index >= p->n_elems)) {
        set_error("parameter index %lld out of range", (long long)index);
        return MG_EINVAL;
    }
    if (kind != MG_PARAM_K0 && index != e) return read_status(p, st);  // no dependence: zero
    MG_CUDA_TRY(cudaMemsetAsync(p->d_tmp, 0, p->n_dofs * sizeof(double), p->stream));
    elem_scatter_kernel<<<1, 64, 0, p->stream>>>(d_sol, p->d_conn, e, p->npe, p->dpn, p->d_tmp);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    if (elast) {
        // f_int is linear in E at a fixed state: d f_e / d rho_e = dE_e f_e(E = 1)
        double lam1, mu1;
        lame_3d(p->mat.nu, lam1, mu1);
        double *Ke = p->d_tmp2;  // 576 doubles
        if (p->physics == MG_PHYSICS_ELASTICITY_HEX8) {
            hex8_kernel<1><<<1, 256, 0, p->stream>>>(p->d_coords, p->d_conn, nullptr, e, 1, p->d_dE,
                                                     nullptr, lam1, mu1, nullptr, nullptr, nullptr, Ke,
                                                     nullptr, nullptr, nullptr, nullptr, st);
            MG_CUDA_TRY(cudaGetLastError());
            elem_matvec_kernel<<<1, 32, 0, p->stream>>>(Ke, p->d_tmp, p->d_conn, e, 1, 8, 3, d_dfe);
        } else {
            hex8_gl_kernel<1><<<1, kGlWarps * 32, 0, p->stream>>>(
                p->d_coords, p->d_conn, nullptr, e, 1, p->d_dE, lam1, mu1, p->d_tmp, nullptr, nullptr,
                nullptr, nullptr, Ke, d_dfe, nullptr, nullptr, nullptr, st);
        }
        MG_CUDA_TRY(cudaGetLastError());
        count_launches(2);
    } else {
        MG_CUDA_TRY(cudaMemsetAsync(p->d_tmp2, 0, p->n_dofs * sizeof(double), p->stream));
        heat_sens_kernel<<<1, 32, 0, p->stream>>>(p->d_coords, p->d_conn, nullptr, e, 1, p->d_tmp,
                                                  p->mat.k0, p->mat.k_beta, p->d_s, p->mat.thickness,
                                                  kind == MG_PARAM_K0 ? 0 : 1, nullptr, nullptr,
                                                  nullptr, p->d_tmp2);
        MG_CUDA_TRY(cudaGetLastError());
        elem_gather_kernel<<<1, 64, 0, p->stream>>>(p->d_tmp2, p->d_conn, e, p->npe, p->dpn, d_dfe);
        MG_CUDA_TRY(cudaGetLastError());
        count_launches(2);
    }
    return read_status(p, st);
}

// m = lumped weights, returned in d_dqdT scaled by 1/area; *qbar = m.T / area
int mean_temperature_terms(mg_problem *p, const double *d_T, double *d_dqdT, double *qbar) {
    MG_CUDA_TRY(cudaMemsetAsync(d_dqdT, 0, p->n_dofs * sizeof(double), p->stream));
    for (int c = 0; c < p->n_colors; c++) {
        int64_t cnt = p->color_ptr[c + 1] - p->color_ptr[c];
        quad4_mass_kernel<<<blocks_for(cnt, 128), 128, 0, p->stream>>>(
            p->d_coords, p->d_conn, p->d_color_elems + p->color_ptr[c], cnt, d_dqdT);
        MG_CUDA_TRY(cudaGetLastError());
    }
    double area = 0, mT = 0;
    // area = sum m (ones vector in d_tmp2)
    std::vector<double> ones(p->n_dofs, 1.0);
    MG_CUDA_TRY(cudaMemcpyAsync(p->d_tmp2, ones.data(), p->n_dofs * sizeof(double),
                                cudaMemcpyHostToDevice, p->stream));
    MG_TRY(dot(p, d_dqdT, p->d_tmp2, p->n_dofs, &area));
    MG_TRY(dot(p, d_dqdT, d_T, p->n_dofs, &mT));
    *qbar = mT / area;
    // scale m by 1/area: reuse dot-free path on host-side factor
    std::vector<double> h(p->n_dofs);
    MG_CUDA_TRY(cudaMemcpyAsync(h.data(), d_dqdT, p->n_dofs * sizeof(double),
                                cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (auto &v : h) v /= area;
    MG_CUDA_TRY(cudaMemcpyAsync(d_dqdT, h.data(), p->n_dofs * sizeof(double),
                                cudaMemcpyHostToDevice, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

}  // namespace mg
