/*
 * ref_driver.cpp -- drives the reference channel kernels compiled for the
 * host (TEST INFRASTRUCTURE ONLY; see ref_build.sh).
 *
 * The kernels themselves come unmodified from the reference sources
 * (collision.cu, streaming.cu, macrovar.cu, BC.cu, LES.cu, globals.cu).  This
 * file supplies what initial.cu and main.cu would: the constant tables
 * (initial.cu:66-178) and the per-step launch sequence (main.cu:360-409,
 * constant-force branch), with every kernel "launch" a loop over the grid.
 */
#include "LBMLES.h"

#include <stdlib.h>
#include <string.h>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
dim3 blockDim(1, 1, 1);
dim3 gridDim(LX, LY, LZ);

template <typename K>
static void launch(K kernel) {
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < LZ; iz++)
        for (int iy = 0; iy < LY; iy++)
            for (int ix = 0; ix < LX; ix++) {
                threadIdx.x = threadIdx.y = threadIdx.z = 0;
                blockIdx.x = ix;
                blockIdx.y = iy;
                blockIdx.z = iz;
                kernel();
            }
}

/* a serial launch over the grid (no OpenMP), for kernels whose threads race */
template <typename K>
static void launch_serial(K kernel) {
    for (int iz = 0; iz < LZ; iz++)
        for (int iy = 0; iy < LY; iy++)
            for (int ix = 0; ix < LX; ix++) {
                threadIdx.x = threadIdx.y = threadIdx.z = 0;
                blockIdx.x = ix;
                blockIdx.y = iy;
                blockIdx.z = iz;
                kernel();
            }
}

extern "C" {

int ref_lx() { return LX; }
int ref_ly() { return LY; }
int ref_lz() { return LZ; }
int ref_use_les() { return USE_LES; }
double ref_tau() { return tau; }
double ref_force_in_x() { return force_in_x; }
double ref_ustar() { return u0; }
double ref_ystar() { return ystar; }

/* constant tables of initial.cu:66-178 */
void ref_init_constants() {
    int h_cix[NPOP] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    int h_ciy[NPOP] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    int h_ciz[NPOP] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    double h_tp[NPOP];
    for (int i = 0; i < NPOP; i++) {
        if (i == 0) h_tp[i] = 8.0 / 27.0;
        else if (i <= 6) h_tp[i] = 2.0 / 27.0;
        else if (i <= 18) h_tp[i] = 1.0 / 54.0;
        else h_tp[i] = 1.0 / 216.0;
    }
    double RT_ = 1.0 / 3.0;
    double cs_ = sqrt(RT_);
    double cs3 = RT_ * cs_;
    for (int i = 0; i < NPOP; i++) {
        d_cix[i] = h_cix[i];
        d_ciy[i] = h_ciy[i];
        d_ciz[i] = h_ciz[i];
        d_tp[i] = h_tp[i];
        d_H100[i] = h_cix[i] / cs_;
        d_H010[i] = h_ciy[i] / cs_;
        d_H001[i] = h_ciz[i] / cs_;
        d_H110[i] = h_cix[i] * h_ciy[i] / RT_;
        d_H101[i] = h_cix[i] * h_ciz[i] / RT_;
        d_H011[i] = h_ciy[i] * h_ciz[i] / RT_;
        d_H200[i] = h_cix[i] * h_cix[i] / RT_ - 1;
        d_H020[i] = h_ciy[i] * h_ciy[i] / RT_ - 1;
        d_H002[i] = h_ciz[i] * h_ciz[i] / RT_ - 1;
        d_H210[i] = h_cix[i] * h_cix[i] * h_ciy[i] / cs3 - h_ciy[i] / cs_;
        d_H201[i] = h_cix[i] * h_cix[i] * h_ciz[i] / cs3 - h_ciz[i] / cs_;
        d_H021[i] = h_ciy[i] * h_ciy[i] * h_ciz[i] / cs3 - h_ciz[i] / cs_;
        d_H120[i] = h_cix[i] * h_ciy[i] * h_ciy[i] / cs3 - h_cix[i] / cs_;
        d_H102[i] = h_cix[i] * h_ciz[i] * h_ciz[i] / cs3 - h_cix[i] / cs_;
        d_H012[i] = h_ciy[i] * h_ciz[i] * h_ciz[i] / cs3 - h_ciy[i] / cs_;
        d_H111[i] = h_cix[i] * h_ciy[i] * h_ciz[i] / cs3;
    }
    d_tau = tau;
    d_ustar = u0;
    d_ystar = ystar;
    d_force_in_x = force_in_x;
    d_pi = pi;
    d_pi2 = pi2;
    d_RT = RT;
    d_cs = cs;
    d_sigma = sigma;
    d_visc = visc;
    d_istep = 1; /* keeps collision_RR's every-1000-steps printf quiet */
}

/* one time step of main.cu:370-409 with the constant force (istep >= 50000
 * branch): forcing, [LES_WALE], collision_RR, streaming, BB, copy back,
 * macrovar, RRBC, macrovar_BN.  All arrays are caller-owned. */
void ref_step(double *f, double *f_temp, double *rho, double *ux, double *uy, double *uz,
              double *fx, double *fy, double *fz, double *taut) {
    launch([&] { forcing(fx, fy, fz); });
    if (USE_LES) launch([&] { LES_WALE(ux, uy, uz, taut); });
    launch([&] { collision_RR(f, fx, fy, fz, rho, ux, uy, uz, taut); });
    launch([&] { streaming(f, f_temp); });
    launch([&] { BB(f, f_temp); });
    memcpy(f, f_temp, sizeof(double) * (size_t)NPOP * LXYZ);
    launch([&] { macrovar(f, fx, fy, fz, rho, ux, uy, uz); });
    launch([&] { RRBC(f, fx, fy, fz, rho, ux, uy, uz, taut); });
    launch([&] { macrovar_BN(f, fx, fy, fz, rho, ux, uy, uz); });
}

void ref_run(int nsteps, double *f, double *f_temp, double *rho, double *ux, double *uy,
             double *uz, double *fx, double *fy, double *fz, double *taut) {
    for (int i = 0; i < nsteps; i++) ref_step(f, f_temp, rho, ux, uy, uz, fx, fy, fz, taut);
}

/* the loop of main.cu:29-46 with the trip forcing: srand(12345) at the start
 * of the run, then for each step n < npforcing the phase redrawn with
 * rand() / RAND_MAX when n % 2000 == 0 and forcing_GP; forcing after */
void ref_run_trip(int nsteps, long long start_istep, int npforcing, double *f, double *f_temp, double *rho,
                  double *ux, double *uy, double *uz, double *fx, double *fy, double *fz, double *taut) {
    srand(12345);
    d_rand_phase = 0.0; /* as at the start of a run (globals.cu), whatever an earlier call left */
    for (long long n = start_istep + 1; n <= start_istep + nsteps; n++) {
        if (n < npforcing) {
            d_istep = (int)n;
            if (n % 2000 == 0) d_rand_phase = (double)rand() / RAND_MAX;
            launch([&] { forcing_GP(fx, fy, fz); });
        } else {
            launch([&] { forcing(fx, fy, fz); });
        }
        d_istep = 1; /* collision_RR prints every 1000 steps otherwise */
        if (USE_LES) launch([&] { LES_WALE(ux, uy, uz, taut); });
        launch([&] { collision_RR(f, fx, fy, fz, rho, ux, uy, uz, taut); });
        launch([&] { streaming(f, f_temp); });
        launch([&] { BB(f, f_temp); });
        memcpy(f, f_temp, sizeof(double) * (size_t)NPOP * LXYZ);
        launch([&] { macrovar(f, fx, fy, fz, rho, ux, uy, uz); });
        launch([&] { RRBC(f, fx, fy, fz, rho, ux, uy, uz, taut); });
        launch([&] { macrovar_BN(f, fx, fy, fz, rho, ux, uy, uz); });
    }
}

/* the step of ref_step with the finite-difference wall closure FDBC in place
 * of RRBC (the alternative main.cu:76-77 leave commented out).  FDBC writes
 * the extrapolated wall velocity and reads its x/z neighbours' in the same
 * kernel, so its result depends on the order of its threads.  Run here so that
 * every neighbour is already extrapolated: a first FDBC over a scratch copy of
 * f leaves the extrapolated wall-row velocities in ux, uy, uz (they depend on
 * rows 1 and 2 only), then FDBC on f rewrites them with the same values and
 * reads only final ones. */
void ref_step_fdbc(double *f, double *f_temp, double *rho, double *ux, double *uy, double *uz,
                   double *fx, double *fy, double *fz, double *taut) {
    launch([&] { forcing(fx, fy, fz); });
    if (USE_LES) launch([&] { LES_WALE(ux, uy, uz, taut); });
    launch([&] { collision_RR(f, fx, fy, fz, rho, ux, uy, uz, taut); });
    launch([&] { streaming(f, f_temp); });
    launch([&] { BB(f, f_temp); });
    memcpy(f, f_temp, sizeof(double) * (size_t)NPOP * LXYZ);
    launch([&] { macrovar(f, fx, fy, fz, rho, ux, uy, uz); });
    launch_serial([&] { FDBC(f_temp, fx, fy, fz, rho, ux, uy, uz, taut); });
    launch_serial([&] { FDBC(f, fx, fy, fz, rho, ux, uy, uz, taut); });
    launch([&] { macrovar_BN(f, fx, fy, fz, rho, ux, uy, uz); });
}

void ref_run_fdbc(int nsteps, double *f, double *f_temp, double *rho, double *ux, double *uy,
                  double *uz, double *fx, double *fy, double *fz, double *taut) {
    for (int i = 0; i < nsteps; i++) ref_step_fdbc(f, f_temp, rho, ux, uy, uz, fx, fy, fz, taut);
}

/* ref_run_trip with FDBC in place of RRBC, run as in ref_step_fdbc */
void ref_run_trip_fdbc(int nsteps, long long start_istep, int npforcing, double *f, double *f_temp, double *rho,
                       double *ux, double *uy, double *uz, double *fx, double *fy, double *fz, double *taut) {
    srand(12345);
    d_rand_phase = 0.0; /* as at the start of a run (globals.cu), whatever an earlier call left */
    for (long long n = start_istep + 1; n <= start_istep + nsteps; n++) {
        if (n < npforcing) {
            d_istep = (int)n;
            if (n % 2000 == 0) d_rand_phase = (double)rand() / RAND_MAX;
            launch([&] { forcing_GP(fx, fy, fz); });
        } else {
            launch([&] { forcing(fx, fy, fz); });
        }
        d_istep = 1; /* collision_RR prints every 1000 steps otherwise */
        if (USE_LES) launch([&] { LES_WALE(ux, uy, uz, taut); });
        launch([&] { collision_RR(f, fx, fy, fz, rho, ux, uy, uz, taut); });
        launch([&] { streaming(f, f_temp); });
        launch([&] { BB(f, f_temp); });
        memcpy(f, f_temp, sizeof(double) * (size_t)NPOP * LXYZ);
        launch([&] { macrovar(f, fx, fy, fz, rho, ux, uy, uz); });
        launch_serial([&] { FDBC(f_temp, fx, fy, fz, rho, ux, uy, uz, taut); });
        launch_serial([&] { FDBC(f, fx, fy, fz, rho, ux, uy, uz, taut); });
        launch([&] { macrovar_BN(f, fx, fy, fz, rho, ux, uy, uz); });
    }
}

/* rand() of this C library after srand(seed), n values (checks of the restatement) */
void ref_rand(unsigned seed, int n, int *out) {
    srand(seed);
    for (int i = 0; i < n; i++) out[i] = rand();
}
}
