/*
 * rr_oracle.h -- CPU restatement (FP64, plain C) of the reference's
 * recursively-regularized lattice-Boltzmann time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product path (the CUDA library behind include/rr_api.h) never links,
 * loads or calls anything in this directory.
 *
 * Every routine follows one reference routine operation by operation (same
 * association of sums and products, same loop order), so that with
 * -ffp-contract=off the results are reproducible bit for bit on any IEEE
 * host.  Citations are path:line inside the reference project.
 *
 * Pinning: the restatement is checked against
 *   - the Taylor-Green golden midline Taylor_Green/RRBMa0.01L100.txt:3-102,
 *   - the reference CUDA channel kernels compiled for the host from their own
 *     sources (oracle/ref_build.sh -> oracle/_ref/), bit for bit.
 */
#ifndef RR_ORACLE_H
#define RR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* velocity orderings */
#define ORC_ORDER_CUDA 0    /* RR27V33_code_DNS_LES/initial.cu:67-69 */
#define ORC_ORDER_FORTRAN 1 /* Taylor_Green/D3Q27RR.f90:69-71, Cavity/para.f90:126-128 */

/* definition of the lattice sound speed */
#define ORC_CS_SQRT_RT 0   /* cs = sqrt(1/3): initial.cu:79-80, Cavity/para.f90:98 */
#define ORC_CS_INV_SQRT3 1 /* cs = 1/sqrt(3): Taylor_Green/D3Q27RR.f90:27 */

/* face kinds, faces ordered x-lo, x-hi, y-lo, y-hi, z-lo, z-hi */
#define ORC_FACE_PERIODIC 0
#define ORC_FACE_WALL 1    /* half-way bounce-back + regularized closure */
#define ORC_FACE_WALL_BB 2 /* half-way bounce-back only */
/* finite-difference wall closure (FDBC, BC.cu:129-309): y faces only, x and z
 * periodic.  Bounce-back as a wall, then every population of the wall node is
 * rebuilt from the extrapolated wall velocity, the finite-difference strain
 * and the density of the known populations (orc_fdbc). */
#define ORC_FACE_FDBC 3

typedef struct {
    int q;   /* 19 or 27 */
    int ord; /* ORC_ORDER_* */
    int cx[27], cy[27], cz[27], opp[27];
    double w[27];
    double rt, cs, cs3;
    double H100[27], H010[27], H001[27];
    double H110[27], H101[27], H011[27], H200[27], H020[27], H002[27];
    double H210[27], H201[27], H021[27], H120[27], H102[27], H012[27], H111[27];
    /* D3Q19 admissible third-order combinations (Taylor_Green/D3Q19RR.f90:131-136) */
    double Hp1[27], Hm1[27], Hp2[27], Hm2[27], Hp3[27], Hm3[27];
} orc_lattice;

typedef struct {
    int nx, ny, nz;
    orc_lattice lat;
    double tau;
    double force[3]; /* uniform body force */
    int les;         /* WALE eddy viscosity on/off */
    double cw;       /* WALE constant */
    int face[6];     /* ORC_FACE_* */
    double uwall[6][3];
    /* Taylor_Green/D3Q27RR.f90 and D3Q19RR.f90 declare their Hermite tables and
     * intermediates as default REAL (D3Q27RR.f90:45-61): with this flag the
     * collision and the start state round them to single precision as that
     * program does; populations, moments and weights stay REAL(8). */
    int tg_real4;
    /* per-node body force (fx, fy, fz: three arrays of nx ny nz), or NULL
     * for the uniform force above */
    const double *ffield;
    /* BGK single-relaxation-time collision of the BGK program instead of the
     * RR one (BGK/collision.cu:3-34), with its incompressible velocity
     * u = sum c f + F/2 (BGK/macrovar.cu:4-31) */
    int bgk;
} orc_params;

/* State in the reference's own form: populations after streaming and wall
 * treatment, the macroscopic fields computed from them, and the eddy
 * viscosity of the last collision.  SoA, f[ip*N + (z*ny + y)*nx + x]. */
typedef struct {
    double *f, *ftmp;
    double *rho, *ux, *uy, *uz, *taut;
} orc_state;

int orc_lattice_init(orc_lattice *L, int q, int order, int cs_mode);

double orc_feq(const orc_lattice *L, int ip, double rho9, double u9, double v9, double w9);

void orc_collide_node(const orc_lattice *L, double tau_eff, const double F[3], double rho9,
                      double u9, double v9, double w9, double *f);
void orc_bgk_node(const orc_lattice *L, double tau, const double F[3], double rho9, double u9, double v9,
                  double w9, double *f);

void orc_regularize_node(const orc_lattice *L, const double F[3], double *f,
                         const int *entering);

void orc_moments_node(const orc_lattice *L, const double F[3], const double *f, double *rho,
                      double *u, double *v, double *w);

/* The finite-difference wall closure of BC.cu:129-309 (the reference launches
 * it in place of RRBC; main.cu:76-77 keep it commented out) on every y face of
 * kind ORC_FACE_FDBC, after the moments of all nodes.  The reference writes the
 * extrapolated wall velocity and reads its x/z neighbours' in one kernel, an
 * order-dependent race; the semantics here are the deterministic ones the
 * kernel's comments state: (1) the wall-row velocity of every column is
 * extrapolated from rows 1 and 2 (BC.cu:148-160), (2) every wall node takes
 * its strain from those velocities, its density from the known populations
 * and rebuilds all of its populations (BC.cu:162-308), (3) the wall-row moments
 * are taken again (macrovar_BN, macrovar.cu:32-59).  taut: the eddy viscosity
 * of the step (NULL for DNS). */
void orc_fdbc(const orc_params *P, double *f, double *rho, double *ux, double *uy, double *uz,
              const double *taut);

/* one full reference time step on the whole grid */
void orc_step(const orc_params *P, orc_state *S);
void orc_run(const orc_params *P, orc_state *S, int nsteps);

/* The channel program's start-up "GP" trip forcing (macrovar.cu:76-115,
 * main.cu:29-46): for steps n < trip_steps the body force is a spatial field
 * of n and of a phase redrawn from the C library's rand() every 2000 steps
 * (srand(12345) at the start of the run, phase 0 before the first draw);
 * from trip_steps on it is the uniform force.  The field's force_in_x is the
 * x component of orc_params.force. */
typedef struct {
    int trip_steps;        /* the reference's npforcing (50000) */
    long long istep;       /* steps done */
    double phase;          /* d_rand_phase */
    int32_t r[34];         /* rand() state: the last 34 terms of its sequence */
    int k;                 /* next slot of r */
    double *fx, *fy, *fz;  /* the force arrays of the current step (caller-owned) */
} orc_trip;

/* the C library's rand() after srand(seed): the additive-feedback generator
 * r_i = r_{i-3} + r_{i-31} (mod 2^32), output r_i >> 1, seeded by
 * r_0 = seed, r_i = 16807 r_{i-1} mod (2^31 - 1) (i < 31), r_i = r_{i-31}
 * (31 <= i < 34), with the first 310 outputs discarded */
void orc_srand(orc_trip *T, unsigned seed);
int orc_rand(orc_trip *T);
/* the force field of step n with phase `phase` into fx, fy, fz */
void orc_trip_force(const orc_params *P, long long n, double phase, double *fx, double *fy, double *fz);
/* nsteps steps with the trip forcing: T->istep advances; before step n the
 * phase is redrawn when n % 2000 == 0 and n < trip_steps */
void orc_run_trip(const orc_params *P, orc_state *S, orc_trip *T, int nsteps);

/* WALE eddy viscosity (LES.cu:4-98), generalised to walls on any face */
void orc_wale(const orc_params *P, const double *ux, const double *uy, const double *uz,
              double *taut);

/* the streaming + wall part of a step, on its own: fin (post-collision) ->
 * fout (post-stream, walls applied); used to check the product's f readout */
void orc_stream_walls(const orc_params *P, const double *fin, double *fout);
void orc_moments_all(const orc_params *P, const double *f, double *rho, double *ux, double *uy,
                     double *uz);
void orc_collide_all(const orc_params *P, double *f, const double *rho, const double *ux,
                     const double *uy, const double *uz, const double *taut);

/* initial states */
void orc_init_tg_reference(const orc_params *P, double U0, double *f, double *rho, double *ux,
                           double *uy, double *uz);
void orc_init_tg_config(const orc_params *P, double U0, double *f, double *rho, double *ux,
                        double *uy, double *uz);
void orc_init_equilibrium2(const orc_params *P, double *f, const double *rho, const double *ux,
                           const double *uy, const double *uz);
void orc_init_channel_loglaw(const orc_params *P, double ustar, double ystar, double *f,
                             double *rho, double *ux, double *uy, double *uz);

/* counter-based random numbers shared with the CUDA library (splitmix64) */
uint64_t orc_splitmix64(uint64_t x);
double orc_uniform_pm1(uint64_t seed, uint64_t node, uint64_t comp);
void orc_init_channel_config(const orc_params *P, double uc, double amp, uint64_t seed,
                             double *f, double *rho, double *ux, double *uy, double *uz);

void orc_set_threads(int n);

/* The reference's file writers (RR27V33_code_DNS_LES/output.cu) restated,
 * writing into directory dir (the reference writes into ./data): fields of
 * n = nx ny nz nodes in the reference layout, f of q n values.  Return 0, or
 * -1 if a file cannot be written.
 *   orc_out_diag     diag_flow (output.cu:3-66): the console line on stdout
 *                    and a line appended to statistics.dat; u0 = the friction
 *                    velocity the console divides umean by
 *   orc_out_flow     output_flow (output.cu:68-140): %09d.dat, rho ux uy uz
 *   orc_out_profile  output_profile (output.cu:142-225): Profiles.txt; the
 *                    reference hands iy + 0.5 to a %d conversion, so its
 *                    first column is whatever integer the variadic call
 *                    leaves there and the eleven %e columns print the first
 *                    eleven doubles; here the first column is iy
 *   orc_out_f        output_f (output.cu:227-258): f%09d.dat */
int orc_out_diag(const char *dir, int istep, long n, const double *rho, const double *ux, const double *uy,
                 const double *uz, double u0);
int orc_out_flow(const char *dir, int istep, long n, const double *rho, const double *ux, const double *uy,
                 const double *uz);
int orc_out_profile(const char *dir, int istep, int nx, int ny, int nz, const double *ux, const double *uy,
                    const double *uz, const double *taut, double ystar);
int orc_out_f(const char *dir, int istep, int q, long n, const double *f);

#ifdef __cplusplus
}
#endif
#endif
