// Runs the device stress-output source of mast-multiphysics_gb300/csrc/hex8_gl.cuh
// on the host, phase by phase over the 32 lanes of a warp, so the CPU tests
// can compare it with the oracle: per Gauss point von Mises, JxW and the KS
// exponential, and sum_qp ex JxW d sigma_vm / d u in var-blocked order.
#include <cmath>

#include "hex8_gl.cuh"

extern "C" int stress_element_host(const double *X, double E, double nu, const double *u_vb, int nonlinear,
                                   double p_ks, double sigma0, double *vm, double *jxw, double *ex,
                                   double *grad) {
    static mg::gl::StressWork s;
    const double lam = E * nu / (1.0 - nu - 2.0 * nu * nu), mu = E / (2.0 * (1.0 + nu));
    for (int a = 0; a < 8; a++)
        for (int c = 0; c < 3; c++) {
            s.X[a * 3 + c] = X[a * 3 + c];
            s.u[a * 3 + c] = u_vb[c * 8 + a];
        }
    bool ok = true;
    for (int lane = 0; lane < 32; lane++) ok = mg::gl::phase_jacobian(s, lane) && ok;
    if (!ok) return -1;
    for (int lane = 0; lane < 32; lane++) mg::gl::phase_gradients(s, lane);
    for (int lane = 0; lane < 32; lane++) mg::gl::phase_von_mises(s, lane, lam, mu, nonlinear != 0, p_ks, sigma0);
    for (int q = 0; q < 8; q++) {
        vm[q] = s.vm[q];
        jxw[q] = s.w[q];
        ex[q] = s.ex[q];
    }
    for (int lane = 0; lane < 24; lane++) grad[(lane % 3) * 8 + lane / 3] = mg::gl::phase_vm_gradient(s, lane);
    return 0;
}
