/* ref_driver_bgk.cpp -- drives the reference's BGK channel kernels
 * (BGK/{collision,streaming,macrovar}.cu, compiled for the host through the
 * shim headers) for the oracle's parity tests.  TEST INFRASTRUCTURE ONLY.
 *
 * It supplies the constant tables of BGK/initial.cu:27-55 and the per-step
 * launch sequence of BGK/main.cu:44-64 with the constant force: forcing,
 * collision_BGK, streaming, streaming2, copy back, macrovar. */
#include <stdlib.h>
#include <string.h>

#include "rb3d.h"

extern double tau, force_in_x, u0, ystar, visc;
extern double pi, pi2;

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
dim3 blockDim(1, 1, 1);

template <class K>
static void launch(K kernel) {
#pragma omp parallel for collapse(3) schedule(static)
    for (int z = 0; z < LZ; z++)
        for (int y = 0; y < LY; y++)
            for (int x = 0; x < LX; x++) {
                threadIdx.x = threadIdx.y = threadIdx.z = 0;
                blockIdx.x = (unsigned)x;
                blockIdx.y = (unsigned)y;
                blockIdx.z = (unsigned)z;
                kernel();
            }
}

extern "C" {

double bgk_tau() { return tau; }
double bgk_force_in_x() { return force_in_x; }

void bgk_init_constants() {
    const int h_cix[NPOP] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    const int h_ciy[NPOP] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    const int h_ciz[NPOP] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    for (int i = 0; i < NPOP; i++) {
        d_cix[i] = h_cix[i];
        d_ciy[i] = h_ciy[i];
        d_ciz[i] = h_ciz[i];
        d_tp[i] = i == 0 ? 8.0 / 27.0 : i <= 6 ? 2.0 / 27.0 : i <= 18 ? 1.0 / 54.0 : 1.0 / 216.0;
    }
    d_tau = tau;
    d_ustar = u0;
    d_ystar = ystar;
    d_force_in_x = force_in_x;
    d_pi = pi;
    d_pi2 = pi2;
    d_visc = visc;
    d_istep = 1;
}

void bgk_run(int nsteps, double *f, double *f_temp, double *rho, double *ux, double *uy, double *uz, double *fx,
             double *fy, double *fz) {
    for (int n = 0; n < nsteps; n++) {
        launch([&] { forcing(fx, fy, fz); });
        launch([&] { collision_BGK(f, fx, fy, fz, rho, ux, uy, uz); });
        launch([&] { streaming(f, f_temp); });
        launch([&] { streaming2(f, f_temp); });
        memcpy(f, f_temp, sizeof(double) * (size_t)NPOP * LXYZ);
        launch([&] { macrovar(f, fx, fy, fz, rho, ux, uy, uz); });
    }
}
}
