// side_loads.cuh -- element side loads, host/device source shared by the
// set-up kernel and the CPU tests (which compile it with g++).
//
//  * HEX8 surface pressure (StructuralElement3D::surface_pressure_residual,
//    src/elasticity/solid_element_3d.cpp:815-876): the residual gets
//    -sum_qp JxW phi_a p n over the side with n the outward normal of the
//    reference configuration, i.e. an external load +int phi_a p n dA.  With
//    the face xi_k = s and tangents t_m = dx/dxi_m, n dA = s (t_k+1 x t_k+2)
//    dxi dxi (Nanson's relation on the reference cube), so no normalisation is
//    needed.  2 x 2 Gauss points on the face, unit weights.
//  * QUAD4 heat flux (HeatConductionElementBase::surface_flux_residual,
//    src/heat_conduction/heat_conduction_elem_base.cpp:876-913): the residual
//    gets +sum_qp JxW phi_a q_n th over the edge, 2 Gauss points.
// Side numbering is libMesh's: HEX8 sides 0..5 are the faces z=-1, y=-1, x=+1,
// y=+1, x=-1, z=+1 of the reference cube; QUAD4 sides 0..3 the edges y=-1,
// x=+1, y=+1, x=-1.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define SL_HD __host__ __device__ __forceinline__
#else
#define SL_HD inline
#endif

namespace mg {
namespace sl {

constexpr double kGauss = 0.57735026918962576451;  // 1/sqrt(3)

// HEX8 node signs in the reference cube (libMesh order)
SL_HD double hex8_node_sign(int a, int m) {
    return m == 0 ? (((a + 1) >> 1 & 1) ? 1.0 : -1.0) : m == 1 ? ((a >> 1 & 1) ? 1.0 : -1.0)
                                                                : ((a >> 2 & 1) ? 1.0 : -1.0);
}

// fixed reference axis and its sign of HEX8 side `side`
SL_HD void hex8_side_axis(int side, int &k, double &s) {
    switch (side) {
        case 0: k = 2; s = -1.0; break;
        case 1: k = 1; s = -1.0; break;
        case 2: k = 0; s = 1.0; break;
        case 3: k = 1; s = 1.0; break;
        case 4: k = 0; s = -1.0; break;
        default: k = 2; s = 1.0; break;
    }
}

// f[3 a + d] += int_side phi_a p n_d dA (node-major element vector)
SL_HD void hex8_pressure_load(const double X[24], int side, double press, double f[24]) {
    int k;
    double s;
    hex8_side_axis(side, k, s);
    const int m1 = (k + 1) % 3, m2 = (k + 2) % 3;
    for (int q = 0; q < 4; q++) {
        double xi[3];
        xi[k] = s;
        xi[m1] = (q & 1) ? kGauss : -kGauss;
        xi[m2] = (q & 2) ? kGauss : -kGauss;
        double N[8], t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
        for (int a = 0; a < 8; a++) {
            const double f0 = 1.0 + hex8_node_sign(a, 0) * xi[0], f1 = 1.0 + hex8_node_sign(a, 1) * xi[1],
                         f2 = 1.0 + hex8_node_sign(a, 2) * xi[2];
            const double fm[3] = {f0, f1, f2};
            N[a] = 0.125 * f0 * f1 * f2;
            // d N_a / d xi_m = sign_m / 8 * product of the other two factors
            const double d1 = 0.125 * hex8_node_sign(a, m1) * fm[k] * fm[m2];
            const double d2 = 0.125 * hex8_node_sign(a, m2) * fm[k] * fm[m1];
            for (int d = 0; d < 3; d++) {
                t1[d] += d1 * X[a * 3 + d];
                t2[d] += d2 * X[a * 3 + d];
            }
        }
        const double c[3] = {s * (t1[1] * t2[2] - t1[2] * t2[1]), s * (t1[2] * t2[0] - t1[0] * t2[2]),
                             s * (t1[0] * t2[1] - t1[1] * t2[0])};
        for (int a = 0; a < 8; a++) {
            const double w = N[a] * press;
            if (w == 0.0) continue;
            for (int d = 0; d < 3; d++) f[a * 3 + d] += w * c[d];
        }
    }
}

// f[a] += int_edge phi_a q_n th ds (QUAD4, nodes (x, y) node-major)
SL_HD void quad4_flux_load(const double X[8], int side, double flux, double th, double f[4]) {
    const int a0 = side, a1 = (side + 1) & 3;  // the edge's two nodes in libMesh order
    const double dx = X[a1 * 2] - X[a0 * 2], dy = X[a1 * 2 + 1] - X[a0 * 2 + 1];
    const double half_len = 0.5 * sqrt(dx * dx + dy * dy);  // JxW of each of the 2 points
    for (int q = 0; q < 2; q++) {
        const double t = q ? kGauss : -kGauss;  // edge coordinate from a0 (-1) to a1 (+1)
        const double n0 = 0.5 * (1.0 - t), n1 = 0.5 * (1.0 + t);
        f[a0] += half_len * n0 * flux * th;
        f[a1] += half_len * n1 * flux * th;
    }
}

}  // namespace sl
}  // namespace mg
