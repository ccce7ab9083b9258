"""Generate the FP64-oracle fixture for the 128x64x64 SIMP cantilever.

Densities: numpy.random.default_rng(0).uniform(0.01, 1.0, 524288), element
order x-fastest.  Runs the oracle (Jacobi-PCG, FP64) twice: to 1e-8 (the
iteration count the CPU baseline extrapolates with) and to 1e-11 (reference
compliance and sensitivities, stored in FP64, for the mixed-precision
error checks).
Writes simp_128x64x64_seed0.npz next to this script.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

NX, NY, NZ, SEED = 128, 64, 64, 0


def main():
    rho = np.random.default_rng(SEED).uniform(0.01, 1.0, NX * NY * NZ)
    t = time.time()
    _, _, r8 = O.simp_solve(O.simp_desc(NX, NY, NZ, rtol=1e-8, maxit=10 ** 6), rho, False)
    t8 = time.time() - t
    t = time.time()
    u, dc, r11 = O.simp_solve(O.simp_desc(NX, NY, NZ, rtol=1e-11, maxit=10 ** 6), rho, True)
    t11 = time.time() - t
    np.savez_compressed(os.path.join(HERE, "simp_128x64x64_seed0.npz"),
                        iterations_1e8=r8.iterations, relres_1e8=r8.relres,
                        compliance_1e8=r8.compliance, iterations_1e11=r11.iterations,
                        relres_1e11=r11.relres, compliance=r11.compliance,
                        dc=dc, u_tip=u[(NX + (NX + 1) * 0) * 3 + 2],
                        threads=O.max_threads(), seconds_1e8=t8, seconds_1e11=t11,
                        t_assemble=r8.t_assemble, t_solve_1e8=r8.t_solve)
    print("1e-8: %d it, C=%.15g (%.1fs); 1e-11: %d it, C=%.15g (%.1fs)"
          % (r8.iterations, r8.compliance, t8, r11.iterations, r11.compliance, t11))


if __name__ == "__main__":
    main()
