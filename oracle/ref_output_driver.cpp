/*
 * ref_output_driver.cpp -- drives the reference's output routines compiled
 * for the host (TEST INFRASTRUCTURE ONLY; see ref_build.sh).
 *
 * RR27V33_code_DNS_LES/output.cu is compiled unmodified: diag_flow,
 * output_flow, output_profile and output_f copy the global device fields
 * (d_rho, d_ux, d_uy, d_uz, d_taut, d_f) to the host arrays and write
 * data/statistics.dat, data/%09d.dat, data/Profiles.txt and data/f%09d.dat
 * under the current directory.  Those globals are globals.cu's; this file
 * points the "device" fields at caller arrays and allocates the host copies
 * (as initialize(), initial.cu:4-19, would), so the test suite can hand the
 * reference's writers the same FP64 fields the library writes.
 */
#include "LBMLES.h"

#include <stdlib.h>

extern "C" {

int ref_out_lx() { return LX; }
int ref_out_ly() { return LY; }
int ref_out_lz() { return LZ; }
double ref_out_ustar() { return u0; }
double ref_out_ystar() { return ystar; }

/* the fields the writers read (LXYZ doubles each; f: NPOP * LXYZ) */
void ref_out_bind(double *rho, double *ux, double *uy, double *uz, double *taut, double *f) {
    d_rho = rho;
    d_ux = ux;
    d_uy = uy;
    d_uz = uz;
    d_taut = taut;
    d_f = f;
    if (!h_rho) {
        h_rho = (double *)malloc(LXYZ * sizeof(double));
        h_ux = (double *)malloc(LXYZ * sizeof(double));
        h_uy = (double *)malloc(LXYZ * sizeof(double));
        h_uz = (double *)malloc(LXYZ * sizeof(double));
        h_taut = (double *)malloc(LXYZ * sizeof(double));
        h_f = (double *)malloc((size_t)NPOP * LXYZ * sizeof(double));
    }
}

void ref_out_diag(int istep) { diag_flow(istep); }
void ref_out_flow(int istep) { output_flow(istep); }
void ref_out_profile(int istep) { output_profile(istep); }
void ref_out_f(int istep) { output_f(istep); }

} /* extern "C" */
