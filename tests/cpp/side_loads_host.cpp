// Runs the device side-load source of mast-multiphysics_gb300/csrc/side_loads.cuh
// on the host for the CPU tests: HEX8 pressure (node-major output) and QUAD4
// heat flux.
#include "side_loads.cuh"

extern "C" void hex8_pressure_host(const double *X, int side, double p, double *f) {
    for (int i = 0; i < 24; i++) f[i] = 0.0;
    mg::sl::hex8_pressure_load(X, side, p, f);
}

extern "C" void quad4_flux_host(const double *X, int side, double flux, double th, double *f) {
    for (int i = 0; i < 4; i++) f[i] = 0.0;
    mg::sl::quad4_flux_load(X, side, flux, th, f);
}
