// Runs the device element source of mast-multiphysics_gb300/csrc/hex8_gl.cuh
// on the host, one phase at a time over the 32 lanes of a warp in the order
// the kernel separates them with __syncwarp(), so the CPU tests can compare
// that exact arithmetic with the oracle.  Output in var-blocked element order
// (dof i 8 + a), the order of mg_element_matrices.
#include "hex8_gl.cuh"

extern "C" int gl_element_host(const double *X, double E, double nu, const double *u_vb,
                               double *f, double *K) {
    static mg::gl::Work s;
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
    for (int lane = 0; lane < 32; lane++) mg::gl::phase_stress(s, lane, lam, mu);
    for (int lane = 0; lane < 32; lane++) mg::gl::phase_projections(s, lane);
    for (int lane = 0; lane < 24; lane++) f[(lane % 3) * 8 + lane / 3] = mg::gl::phase_force(s, lane);
    for (int lane = 0; lane < 32; lane++)
        for (int h = 0; h < 2; h++) {
            const int p = lane + 32 * h, a = p >> 3, b = p & 7;
            double Kb[9];
            mg::gl::phase_tangent(s, a, b, lam, mu, Kb);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) K[(i * 8 + a) * 24 + j * 8 + b] = Kb[i * 3 + j];
        }
    return 0;
}
