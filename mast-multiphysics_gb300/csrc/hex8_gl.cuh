// hex8_gl.cuh -- geometrically nonlinear (total Lagrangian, Green-Lagrange
// strain) HEX8 element, the NONLINEAR_STRAIN branch of
// StructuralElement3D::internal_residual (src/elasticity/solid_element_3d.cpp:
// 299-409, strain operator initialize_green_lagrange_strain_operator :1309-1463)
// with the isotropic St Venant-Kirchhoff material of
// IsotropicMaterialProperty::StiffnessMatrix3D
// (src/property_cards/isotropic_material_property_card.cpp:512-528).
//
// Written per node pair instead of with the reference's 6 x 24 strain
// operators.  With Fd = I + grad u (rows f_i) and physical shape gradients g_a,
// the strain variation of dof (component i, node a) is sym(f_i (x) g_a), so
//   internal force   f_ia = sum_qp JxW (Fd S g_a)_i
//   material tangent K_ia,jb = sum_qp JxW [lam (f_i.g_a)(f_j.g_b)
//                                  + mu ((f_i.f_j)(g_a.g_b) + (f_i.g_b)(f_j.g_a))]
//   geometric        + delta_ij sum_qp JxW g_a.S.g_b
// with S = lam tr(E) I + 2 mu E, E = (Fd^T Fd - I)/2 (the second Piola-Kirchhoff
// stress of C applied to the Green-Lagrange strain in Voigt form).
//
// One warp evaluates one element.  The work is split into phases over a
// per-warp workspace; a phase is a function of the lane index, and lanes only
// read what earlier phases wrote, so the kernel separates phases by
// __syncwarp() and a host loop over the 32 lanes runs the same source.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define GL_HD __host__ __device__ __forceinline__
#else
#define GL_HD inline
#endif

namespace mg {
namespace gl {

// element workspace of one warp (doubles; 924 = 7.4 KB)
struct Work {
    double X[24];        // node coordinates, node-major (3 a + d)
    double u[24];        // displacements, node-major (3 a + c)
    double w[8];         // JxW per Gauss point (unit weights)
    double inv[8][9];    // inverse Jacobian per Gauss point
    double g[8][8][3];   // physical gradients g[q][a]
    double Fd[8][9];     // deformation gradient I + grad u per Gauss point
    double S[8][9];      // second Piola-Kirchhoff stress (symmetric, full 3 x 3)
    double B[8][9];      // Fd Fd^T (f_i . f_j)
    double Fg[8][8][3];  // Fd g_a  (f_i . g_a)
    double Sg[8][8][3];  // S g_a
};

constexpr double kGauss = 0.57735026918962576451;  // 1/sqrt(3)

// reference gradient of shape function a at Gauss point q = i + 2 j + 4 k
// (libMesh HEX8 node order: x signs - + + -, y signs - - + +, z - for nodes 0-3)
GL_HD void dref(int q, int a, double d[3]) {
    const double xi = (q & 1) ? kGauss : -kGauss, eta = (q >> 1 & 1) ? kGauss : -kGauss,
                 zeta = (q >> 2 & 1) ? kGauss : -kGauss;
    const double sx = ((a + 1) >> 1 & 1) ? 1.0 : -1.0, sy = (a >> 1 & 1) ? 1.0 : -1.0,
                 sz = (a >> 2 & 1) ? 1.0 : -1.0;
    const double fx = 0.5 * (1.0 + sx * xi), fy = 0.5 * (1.0 + sy * eta), fz = 0.5 * (1.0 + sz * zeta);
    d[0] = 0.5 * sx * fy * fz;
    d[1] = 0.5 * sy * fx * fz;
    d[2] = 0.5 * sz * fx * fy;
}

// phase 1 (lanes 0-7, q = lane): Jacobian, JxW, inverse.  Returns false for a
// non-positive determinant.  (W: any workspace with X, w, inv.)
template <class W>
GL_HD bool phase_jacobian(W &s, int lane) {
    if (lane >= 8) return true;
    const int q = lane;
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // J[i][j] = d x_j / d xi_i
    for (int a = 0; a < 8; a++) {
        double d[3];
        dref(q, a, d);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) J[i * 3 + j] += d[i] * s.X[a * 3 + j];
    }
    const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                       J[2] * (J[3] * J[7] - J[4] * J[6]);
    double *iv = s.inv[q];
    iv[0] = (J[4] * J[8] - J[5] * J[7]) / det;
    iv[1] = (J[2] * J[7] - J[1] * J[8]) / det;
    iv[2] = (J[1] * J[5] - J[2] * J[4]) / det;
    iv[3] = (J[5] * J[6] - J[3] * J[8]) / det;
    iv[4] = (J[0] * J[8] - J[2] * J[6]) / det;
    iv[5] = (J[2] * J[3] - J[0] * J[5]) / det;
    iv[6] = (J[3] * J[7] - J[4] * J[6]) / det;
    iv[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    iv[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    s.w[q] = det;
    return det > 0.0;
}

// phase 2 (every lane, (q, a) = (p >> 3, p & 7) for p = lane, lane + 32):
// physical gradients g_j = sum_k (d xi_k / d x_j) d phi / d xi_k
template <class W>
GL_HD void phase_gradients(W &s, int lane) {
    for (int h = 0; h < 2; h++) {
        const int p = lane + 32 * h, q = p >> 3, a = p & 7;
        double d[3];
        dref(q, a, d);
        const double *iv = s.inv[q];
        for (int j = 0; j < 3; j++) s.g[q][a][j] = iv[j * 3] * d[0] + iv[j * 3 + 1] * d[1] + iv[j * 3 + 2] * d[2];
    }
}

// phase 3 (lanes 0-7, q = lane): Fd, Green-Lagrange strain, S, Fd Fd^T.  The
// strain is formed from H = grad u as (H + H^T + H^T H) / 2, not as
// (Fd^T Fd - I) / 2, whose subtraction would cancel the leading digits of small
// strains (a 1e-8 strain would keep only 8 significant digits).
GL_HD void phase_stress(Work &s, int lane, double lam, double mu) {
    if (lane >= 8) return;
    const int q = lane;
    double H[9], Fd[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double v = 0.0;
            for (int a = 0; a < 8; a++) v += s.u[a * 3 + i] * s.g[q][a][j];
            H[i * 3 + j] = v;
            Fd[i * 3 + j] = v + (i == j ? 1.0 : 0.0);
        }
    double E[9];
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) {
            double c = 0.0;
            for (int m = 0; m < 3; m++) c += H[m * 3 + j] * H[m * 3 + k];
            E[j * 3 + k] = 0.5 * (H[j * 3 + k] + H[k * 3 + j] + c);
        }
    const double tr = E[0] + E[4] + E[8];
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) {
            s.S[q][j * 3 + k] = 2.0 * mu * E[j * 3 + k] + (j == k ? lam * tr : 0.0);
            double b = 0.0;
            for (int m = 0; m < 3; m++) b += Fd[j * 3 + m] * Fd[k * 3 + m];
            s.B[q][j * 3 + k] = b;
            s.Fd[q][j * 3 + k] = Fd[j * 3 + k];
        }
}

// phase 4 (every lane, (q, a) as in phase 2): Fd g_a and S g_a
GL_HD void phase_projections(Work &s, int lane) {
    for (int h = 0; h < 2; h++) {
        const int p = lane + 32 * h, q = p >> 3, a = p & 7;
        const double *g = s.g[q][a];
        for (int i = 0; i < 3; i++) {
            s.Fg[q][a][i] = s.Fd[q][i * 3] * g[0] + s.Fd[q][i * 3 + 1] * g[1] + s.Fd[q][i * 3 + 2] * g[2];
            s.Sg[q][a][i] = s.S[q][i * 3] * g[0] + s.S[q][i * 3 + 1] * g[1] + s.S[q][i * 3 + 2] * g[2];
        }
    }
}

// phase 5a (lanes 0-23, lane = 3 a + i): internal force of dof (i, a)
GL_HD double phase_force(const Work &s, int lane) {
    const int a = lane / 3, i = lane % 3;
    double f = 0.0;
    for (int q = 0; q < 8; q++) {
        const double *Fd = s.Fd[q] + i * 3;
        const double *Sg = s.Sg[q][a];
        f += s.w[q] * (Fd[0] * Sg[0] + Fd[1] * Sg[1] + Fd[2] * Sg[2]);
    }
    return f;
}

// phase 5b (node pair (a, b)): the 3 x 3 tangent block K[i][j] = K_ia,jb
GL_HD void phase_tangent(const Work &s, int a, int b, double lam, double mu, double K[9]) {
    for (int k = 0; k < 9; k++) K[k] = 0.0;
    for (int q = 0; q < 8; q++) {
        const double *ga = s.g[q][a], *gb = s.g[q][b];
        const double *Fa = s.Fg[q][a], *Fb = s.Fg[q][b];
        const double wq = s.w[q];
        const double gab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
        const double gsg = ga[0] * s.Sg[q][b][0] + ga[1] * s.Sg[q][b][1] + ga[2] * s.Sg[q][b][2];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double k = lam * Fa[i] * Fb[j] + mu * (s.B[q][i * 3 + j] * gab + Fb[i] * Fa[j]);
                if (i == j) k += gsg;
                K[i * 3 + j] += wq * k;
            }
    }
}

// ---------------------------------------------------------------------------
// Stress output (StructuralElement3D::calculate_stress, solid_element_3d.cpp:
// 1147-1270; von Mises and its derivatives, stress_output_base.cpp:183-271;
// the KS weights of ks_stress_output.cpp:41-99).  Per Gauss point: the strain
// (linear: B u; nonlinear: the Green-Lagrange strain), sigma = C eps with the
// stress modulus, sigma_vm, ex = exp(p (sigma_vm - s0) / s0), and the tensor T
// of t = C (d sigma_vm / d sigma) (T_jj = t_j, off-diagonal = the shear entry),
// so that d sigma_vm / d u_ia = (Fd T g_a)_i with Fd = I (linear) or I + grad u.
// ---------------------------------------------------------------------------
struct StressWork {
    double X[24], u[24], w[8], inv[8][9], g[8][8][3];
    double Fd[8][9];
    double T[8][9];
    double vm[8];
    double ex[8];
};

// lanes 0-7, q = lane
GL_HD void phase_von_mises(StressWork &s, int lane, double lam, double mu, bool nonlinear,
                           double p_ks, double sigma0) {
    if (lane >= 8) return;
    const int q = lane;
    double H[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double v = 0.0;
            for (int a = 0; a < 8; a++) v += s.u[a * 3 + i] * s.g[q][a][j];
            H[i * 3 + j] = v;
            s.Fd[q][i * 3 + j] = (nonlinear ? v : 0.0) + (i == j ? 1.0 : 0.0);
        }
    // Voigt strain [xx, yy, zz, xy, yz, zx], engineering shears
    static constexpr int VJ[6] = {0, 1, 2, 0, 1, 0}, VK[6] = {0, 1, 2, 1, 2, 2};
    double eps[6];
    for (int r = 0; r < 6; r++) {
        const int j = VJ[r], k = VK[r];
        double e = (r < 3) ? H[j * 3 + j] : H[j * 3 + k] + H[k * 3 + j];
        if (nonlinear) {
            double c = 0.0;
            for (int m = 0; m < 3; m++) c += H[m * 3 + j] * H[m * 3 + k];
            e += (r < 3) ? 0.5 * c : c;
        }
        eps[r] = e;
    }
    const double tr = eps[0] + eps[1] + eps[2];
    double sg[6];
    for (int r = 0; r < 3; r++) sg[r] = lam * tr + 2.0 * mu * eps[r];
    for (int r = 3; r < 6; r++) sg[r] = mu * eps[r];
    const double P = 0.5 * ((sg[0] - sg[1]) * (sg[0] - sg[1]) + (sg[1] - sg[2]) * (sg[1] - sg[2]) +
                            (sg[2] - sg[0]) * (sg[2] - sg[0])) +
                     3.0 * (sg[3] * sg[3] + sg[4] * sg[4] + sg[5] * sg[5]);
    const double vm = sqrt(P);
    double d[6] = {0, 0, 0, 0, 0, 0};  // d sigma_vm / d sigma, zero where sigma_vm = 0
    if (P > 0.0) {
        const double c = 0.5 / vm;
        d[0] = c * (2.0 * sg[0] - sg[1] - sg[2]);
        d[1] = c * (2.0 * sg[1] - sg[2] - sg[0]);
        d[2] = c * (2.0 * sg[2] - sg[0] - sg[1]);
        for (int r = 3; r < 6; r++) d[r] = c * 6.0 * sg[r];
    }
    const double trd = d[0] + d[1] + d[2];
    double *T = s.T[q];
    T[0] = lam * trd + 2.0 * mu * d[0];
    T[4] = lam * trd + 2.0 * mu * d[1];
    T[8] = lam * trd + 2.0 * mu * d[2];
    T[1] = T[3] = mu * d[3];
    T[5] = T[7] = mu * d[4];
    T[2] = T[6] = mu * d[5];
    s.vm[q] = vm;
    s.ex[q] = exp(p_ks * (vm - sigma0) / sigma0);
}

// lanes 0-23, lane = 3 a + i: sum_qp ex JxW d sigma_vm / d u_ia
GL_HD double phase_vm_gradient(const StressWork &s, int lane) {
    const int a = lane / 3, i = lane % 3;
    double acc = 0.0;
    for (int q = 0; q < 8; q++) {
        const double *g = s.g[q][a], *T = s.T[q], *F = s.Fd[q] + i * 3;
        double Tg[3];
        for (int m = 0; m < 3; m++) Tg[m] = T[m * 3] * g[0] + T[m * 3 + 1] * g[1] + T[m * 3 + 2] * g[2];
        acc += s.w[q] * s.ex[q] * (F[0] * Tg[0] + F[1] * Tg[1] + F[2] * Tg[2]);
    }
    return acc;
}

}  // namespace gl
}  // namespace mg
