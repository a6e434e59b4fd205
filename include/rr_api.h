/*
 * rr_api.h -- C ABI of the GB300 recursively-regularized lattice-Boltzmann
 * solver (librrlbm.so).  Plain pointers and sizes only.
 *
 * It replaces the host loop of the reference CUDA channel code,
 * RR27V33_code_DNS_LES/main.cu:31-117, whose body calls the kernels declared
 * in RR27V33_code_DNS_LES/LBMLES.h:60-81 on global device arrays and then the
 * output routines of LBMLES.h:83-86.  With this library that loop becomes
 *
 *     rr_params p; rr_params_default(&p);  ... set knobs ...
 *     rr_solver *s; rr_create(&p, &s);
 *     rr_init_state(s, f, rho, ux, uy, uz, RR_HOST);      // initialize()
 *     for (istep = 1; istep <= NEND; istep++) {
 *         rr_step(s, 1);                                  // main.cu:360-409
 *         if (istep % NDIAG == 0) rr_output(s, RR_OUT_DIAG, "data");
 *         ...
 *     }
 *     rr_destroy(s);
 *
 * Every function returns an rr_status and never exits the process; the text
 * of the last error of the calling thread is available from rr_last_error().
 * All device work of a solver runs on that solver's own CUDA stream;
 * rr_step() only enqueues work, rr_sync() waits for it and reports the
 * device-side watchdog (density out of range or NaN).
 */
#ifndef RR_API_H
#define RR_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    RR_OK = 0,
    RR_ERR_INVALID = 1,     /* bad argument or parameter */
    RR_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    RR_ERR_NOMEM = 3,       /* device or host allocation failed */
    RR_ERR_UNSUPPORTED = 4, /* combination not built */
    RR_ERR_WATCHDOG = 5,    /* density left (0.1, 10) or became NaN, or a bounded
                               wait of the staged step gave up (rr_last_error says which) */
    RR_ERR_IO = 6,          /* file could not be opened / read / written */
    RR_ERR_STATE = 7        /* call out of order (e.g. step before init) */
} rr_status;

/* population storage in HBM; arithmetic is FP64 for RR_STORE_F64, FP32 else */
typedef enum { RR_STORE_F64 = 0, RR_STORE_F32 = 1, RR_STORE_F16 = 2, RR_STORE_BF16 = 3 } rr_storage;

/* face kinds; faces are ordered x-lo, x-hi, y-lo, y-hi, z-lo, z-hi */
typedef enum {
    RR_FACE_PERIODIC = 0,
    RR_FACE_WALL = 1,    /* half-way bounce-back + regularized closure (RRBC) */
    RR_FACE_WALL_BB = 2, /* half-way bounce-back only */
    /* finite-difference wall closure (FDBC, RR27V33_code_DNS_LES/BC.cu:129-309,
     * the alternative main.cu:76-77 leave commented out): y faces only, x and
     * z periodic, wall at rest, ly >= 4, RR collision.  Every population of
     * the wall node is rebuilt from the wall velocity extrapolated from rows
     * 1 and 2 inward, the finite-difference strain and the density of the
     * populations streamed in from inside.  The velocities of all wall nodes
     * are extrapolated before any closure reads its neighbours' (the
     * reference's single kernel races there).  With WALE: the two-pass method
     * only (lx >= 3). */
    RR_FACE_FDBC = 3
} rr_face;

/* velocity ordering of populations crossing the API (rr_init_state, rr_get_f,
 * rr_save / rr_load):  RR_ORDER_CUDA = RR27V33_code_DNS_LES/initial.cu:67-69,
 * RR_ORDER_FORTRAN = Taylor_Green/D3Q27RR.f90:69-71 = Cavity/para.f90:126-128
 * (the only ordering defined for D3Q19, Taylor_Green/D3Q19RR.f90:75-77) */
typedef enum { RR_ORDER_CUDA = 0, RR_ORDER_FORTRAN = 1 } rr_order;

/* rounding of FP16/BF16 population stores (no effect on FP32/FP64 storage):
 * stochastic rounding is unbiased, so population changes smaller than half a
 * unit in the last place accumulate instead of stalling */
typedef enum { RR_ROUND_NEAREST = 0, RR_ROUND_STOCHASTIC = 1 } rr_rounding;

/* where a caller buffer lives */
typedef enum { RR_HOST = 0, RR_DEVICE = 1 } rr_where;

/* rr_output() selectors: the reference's four outputs (output.cu) */
#define RR_OUT_DIAG 1u    /* diag_flow: console line + data/statistics.dat (output.cu:3-66) */
#define RR_OUT_FLOW 2u    /* output_flow: data/%09d.dat rho,ux,uy,uz FP64 (output.cu:68-140) */
#define RR_OUT_PROFILE 4u /* output_profile: data/Profiles.txt (output.cu:142-225) */
#define RR_OUT_F 8u       /* output_f: data/f%09d.dat, 27 N FP64 (output.cu:227-258) */

/* Run-time counterpart of parameters.h:1-25 and globals.cu:18-40. */
typedef struct rr_params {
    int lx, ly, lz;      /* LX, LY, LZ (parameters.h:9-11) */
    int q;               /* NPOP: 27, or 19 (Taylor_Green/D3Q19RR.f90) */
    int use_les;         /* USE_LES (parameters.h:6): WALE eddy viscosity */
    double tau;          /* relaxation time, tau = 3 nu + 0.5 (globals.cu:36) */
    double cw;           /* WALE constant (LES.cu:12) */
    double force[3];     /* uniform body force; force_in_x = 2 u*^2 / LY (globals.cu:38) */
    int face[6];         /* rr_face of x-lo, x-hi, y-lo, y-hi, z-lo, z-hi */
    double uwall[6][3];  /* velocity of each wall face (moving lid, Cavity/streaming.f90:142-152) */
    int storage;         /* rr_storage */
    int order;           /* rr_order of populations crossing the API */
    int device;          /* CUDA device ordinal */
    double ustar, ystar; /* friction velocity and viscous length, for output_profile's y+ */
    int rounding;        /* rr_rounding of FP16/BF16 stores (default stochastic) */
    /* start-up trip forcing of the channel program (forcing_GP,
     * macrovar.cu:76-115; main.cu:29-46): for time steps n < trip_steps the
     * body force is its spatial field of n and of a phase redrawn from the C
     * library's rand() sequence (srand(12345) at the start of the run) every
     * 2000 steps, with force[0] as force_in_x; from trip_steps on the uniform
     * force.  0 (default): off; the reference's value is 50000.  D3Q27 and
     * lx >= 3 only; steps in the trip phase run without CUDA graphs. */
    int trip_steps;
    /* rr_collision: the RR collision (default), or the BGK program's
     * single-relaxation-time collision with its incompressible velocity
     * u = sum c f + F/2 (BGK/collision.cu:3-34, BGK/macrovar.cu:4-31); BGK
     * needs D3Q27, DNS, lx >= 3, bounce-back walls without the regularized
     * closure (RR_FACE_WALL_BB) and no trip forcing */
    int collision;
} rr_params;

typedef enum { RR_COLL_RR = 0, RR_COLL_BGK = 1 } rr_collision;

typedef struct rr_solver rr_solver;

/* The defaults of parameters.h / globals.cu: 64^3 Re_tau = 180 channel, DNS,
 * walls at y = 0 and y = LY-1, periodic x and z, nu = 0.000622,
 * u* = 2 Re_tau nu / LY, tau = 3 nu + 0.5, F_x = 2 u*^2 / LY, D3Q27, FP64. */
rr_status rr_params_default(rr_params *p);

/* allocation of device state: initialize() (initial.cu:4-19) */
rr_status rr_create(const rr_params *p, rr_solver **out);
rr_status rr_destroy(rr_solver *s);

/* Sets the state the reference holds before its first step: post-stream
 * populations f (NPOP x N FP64, f[ip * N + (z * LY + y) * LX + x], in
 * p->order) and the macroscopic fields the first collision uses
 * (init_arrays, initial.cu:268-326, and the CONTINUE_STEP restart,
 * initial.cu:189-265).  f may be NULL: the second-order equilibrium of
 * (rho, u) is used (Cavity/initial.f90:3-34).  Resets the step counter.
 * With RR_HOST the call returns once the host arrays are copied (the caller
 * may reuse them); the upload and first collision run on, in order on the
 * solver's stream. */
rr_status rr_init_state(rr_solver *s, const double *f, const double *rho, const double *ux,
                        const double *uy, const double *uz, int where);

/* nsteps full time steps (main.cu:360-409), one fused kernel each, enqueued
 * on the solver's stream (CUDA graphs for long runs). */
rr_status rr_step(rr_solver *s, int nsteps);
rr_status rr_sync(rr_solver *s);
/* Whether the solver's work is still in flight: *busy = 1 while enqueued
 * steps, uploads or readouts have not finished on its stream, 0 once they
 * have.  Never waits and does not read the watchdog (rr_sync does).  No
 * counterpart in the reference, whose host loop synchronises every kernel;
 * a server polls it to advance each resident domain at its own pace. */
rr_status rr_query(rr_solver *s, int *busy);
long long rr_get_istep(const rr_solver *s);
/* the solver's CUDA stream (a cudaStream_t), for callers that order their own
 * work or CUDA events against the solver's; no counterpart in the reference,
 * which runs everything on the default stream (main.cu:381-409) */
void *rr_get_stream(const rr_solver *s);

/* Macroscopic fields after the last step, what the reference holds in
 * d_rho, d_ux, d_uy, d_uz (FP64, N each).  taut (may be NULL) receives the
 * WALE eddy viscosity tau_t = 3 nu_t of those fields, i.e. the one the next
 * collision uses.  Any pointer may be NULL. */
rr_status rr_macro(rr_solver *s, double *rho, double *ux, double *uy, double *uz, double *taut,
                   int where);

/* Post-stream populations after the last step (d_f after main.cu:64 and the
 * wall closure), FP64, NPOP x N, in p->order. */
rr_status rr_get_f(rr_solver *s, double *f, int where);

/* diag_flow's statistics (output.cu:24-35): {umean, vmean, wmean, rhomean} */
rr_status rr_diag(rr_solver *s, double out[4]);

/* The same four means of FP64 fields that already live on the device (n
 * values each), written to the device array out[4] on `stream` (a
 * cudaStream_t, NULL for the default stream), without allocating anything.
 * No counterpart in the reference.  It is for callers that may not allocate
 * device memory when they ask for the statistics: a server whose HBM budget
 * is fully handed out to resident domains, or a latency-critical loop that
 * cannot afford a cudaMalloc.  The partial sums use a fixed 32 KiB array that
 * every GPU loading the library holds until the process exits; n must be 1 to
 * 2147483647.  The first call on a device looks up that array's device
 * address (with the device current), so make it before any stream capture.
 * Calls share the array: two calls that overlap on the GPU race.  Nothing is
 * synchronised; read out[] after the stream's work completes.  The looked-up
 * address is kept for the life of the process: after a cudaDeviceReset() of a
 * device the library's device memory there is gone, so do not call this
 * function on that device again in the same process. */
rr_status rr_diag_fields_noalloc(const double *rho, const double *ux, const double *uy,
                                 const double *uz, size_t n, double *out, void *stream);

/* output_profile's statistics per y plane (output.cu:181-214), FP64 on the
 * device: out[iy * 11 + k] for k = y+0.5, (y+0.5)/ystar, <u>, <v>, <w>,
 * <u'u'>, <v'v'>, <w'w'>, <u'v'>, <u'w'>, <v'w'>, and out[LY*11 + iy] = <tau_t>
 * (out must hold 12 * LY doubles). */
rr_status rr_profile(rr_solver *s, double *out);

/* Time-averaging accumulators (FP64, on the device): rr_accumulate() adds the
 * current y-plane profile (12 * LY values, as rr_profile) to the running sums;
 * rr_get_accum() returns the sums and the number of samples. */
rr_status rr_accumulate(rr_solver *s);
rr_status rr_get_accum(rr_solver *s, double *sums, long long *samples);

/* The reference's file outputs, byte-compatible (what = RR_OUT_* bits),
 * written under directory dir with istep = rr_get_istep(). */
rr_status rr_output(rr_solver *s, unsigned what, const char *dir);

/* The body force of the step the readouts show (the reference's
 * d_force_realx/y/z, LBMLES.h:46-50, written by forcing / forcing_GP):
 * fx, fy, fz of n values each, consecutively in out (3 n doubles), on the
 * host or the device.  The uniform force outside the trip-forcing phase. */
rr_status rr_get_force(rr_solver *s, double *out, int where);

/* Restart files in the reference's format (output_flow + output_f, read
 * back by initialize() with CONTINUE_STEP, initial.cu:189-265):
 * dir/%09d.dat and dir/f%09d.dat. */
rr_status rr_save(rr_solver *s, const char *dir);
rr_status rr_load(rr_solver *s, const char *dir, long long istep);

/* memory the solver holds on the device, in bytes */
size_t rr_device_bytes(const rr_solver *s);
/* bytes a solver with these parameters would hold (admission control) */
size_t rr_bytes_for(const rr_params *p);

/* text of the last error on this thread ("" if none) */
const char *rr_last_error(void);

/* ---- Batches: many domains advanced together ------------------------------
 * No counterpart in the reference, which runs one domain per process.  A
 * batch steps every member solver in one persistent kernel launch per step
 * (per storage type / lattice / forcing class; WALE members and grids with
 * lx < 3 add their own launch), captured in CUDA graphs of 32 steps.  Each
 * member's nodes get exactly the arithmetic of the member's own rr_step, so
 * its results are the same alone and in a batch.
 *
 * While a solver is a member, its work runs on the batch's stream
 * (rr_get_stream returns that stream); rr_macro, rr_get_f, rr_diag, rr_profile,
 * rr_accumulate, rr_output and rr_save work as before, while rr_step,
 * rr_init_state and rr_load return RR_ERR_STATE.  rr_destroy of a member
 * removes it first. */
typedef struct rr_batch rr_batch;

rr_status rr_batch_create(int device, rr_batch **out);
/* removes every member (waiting for the batch's work), then frees the batch */
rr_status rr_batch_destroy(rr_batch *b);
/* s must have a state (rr_init_state / rr_load), live on the batch's device
 * and belong to no other batch */
rr_status rr_batch_add(rr_batch *b, rr_solver *s);
rr_status rr_batch_remove(rr_batch *b, rr_solver *s);
int rr_batch_size(const rr_batch *b);
/* advance every member by nsteps (enqueued on the batch's stream) */
rr_status rr_batch_step(rr_batch *b, int nsteps);
/* wait for the batch's work; RR_ERR_WATCHDOG if a member's watchdog fired
 * (rr_last_error names the member, in order of addition) */
rr_status rr_batch_sync(rr_batch *b);
void *rr_batch_get_stream(const rr_batch *b);
/* launch shape of the persistent kernel: threads per CTA (64, 128 or 256),
 * resident CTAs per SM (0: the kernel's occupancy limit) and the order in
 * which the persistent CTAs walk the members' CTAs */
typedef enum { RR_BATCH_STRIDED = 0, RR_BATCH_CHUNKED = 1 } rr_batch_order;
rr_status rr_batch_set_launch(rr_batch *b, int block, int ctas_per_sm, int order);
rr_status rr_batch_get_launch(const rr_batch *b, int *block, int *ctas_per_sm, int *order);
/* how a step of the batch is launched: RR_BATCH_PERSISTENT, one persistent
 * batch kernel per class (above); RR_BATCH_FANOUT, each member's own step
 * launches, the members spread over `chains` parallel branches of the graph
 * (largest first to the least loaded branch), a branch running its members'
 * steps member after member.  Same results either way. */
typedef enum { RR_BATCH_PERSISTENT = 0, RR_BATCH_FANOUT = 1 } rr_batch_mode;
rr_status rr_batch_set_mode(rr_batch *b, int mode, int chains);
rr_status rr_batch_get_mode(const rr_batch *b, int *mode, int *chains);
/* L2 grouping: members whose population buffers fit are packed (in order of
 * addition, per class) into groups of at most group_bytes, and each group
 * runs its steps of an rr_batch_step back to back, so its data stays in L2
 * across steps; larger members share one launch per step.  0 turns grouping
 * off (the default). */
rr_status rr_batch_set_grouping(rr_batch *b, size_t group_bytes);
size_t rr_batch_get_grouping(const rr_batch *b);

/* ---- Autotuner ------------------------------------------------------------
 * No counterpart in the reference (its launch shapes are the compile-time
 * BLOCK_* of parameters.h).  Tries launch shapes on the solver's (or batch's)
 * real steps, each for trial_steps steps timed with CUDA events, keeps the
 * fastest and records it for the size class (lattice, storage, WALE, force,
 * node count rounded to a power of two); solvers created later in that class
 * start with it.  The shapes change no result, so the trial steps are
 * ordinary steps: the state advances by (number of candidates) * trial_steps
 * (reported in *steps_run).  Tile step and two-pass WALE step: rows per
 * work-item group; DNS: tile or staged step, the staged block rows and
 * stages; fused WALE step: the x-y tile and z chunk (the WALE method
 * itself is not tuned: the two methods round differently); batch: the mode
 * (fan-out chains 4, 8, 16 or the persistent kernel), threads per CTA, CTAs per
 * SM, walk order, L2 grouping and the rows per group of each size class
 * present.  Synchronises. */
rr_status rr_tune(rr_solver *s, int trial_steps, long long *steps_run);
/* the solver's launch shapes: rows per work-item group of the tile step (a
 * multiple of 32); the WALE step's method (RR_LES_FUSED: one launch of
 * z-marching tiles {tx, ty, z chunk} with a shared-memory velocity ring;
 * RR_LES_TWO_PASS: two tile-step launches through a velocity field, lx >= 3);
 * les_method and les_tile may be NULL */
typedef enum { RR_LES_FUSED = 0, RR_LES_TWO_PASS = 1 } rr_les_method;
rr_status rr_get_launch(const rr_solver *s, int *rows_group, int *les_method, int les_tile[3]);
rr_status rr_set_launch(rr_solver *s, int rows_group, const int *les_method, const int les_tile[3]);
rr_status rr_batch_tune(rr_batch *b, int trial_steps, long long *steps_run);
/* the DNS step's method: RR_DNS_TILE, one launch of warp work items (any
 * grid with lx >= 3); RR_DNS_STAGED, rows on a y/z face in one launch and the
 * interior rows in blocks of `rows` rows through a `stages`-deep pipeline of
 * bulk copies into shared memory (DNS, lx, ly, lz >= 3, lx times the element
 * size a multiple of 16 bytes).  Same results bit for bit. */
typedef enum { RR_DNS_TILE = 0, RR_DNS_STAGED = 1 } rr_dns_method;
rr_status rr_set_stage(rr_solver *s, int method, int rows, int stages);
rr_status rr_get_stage(const rr_solver *s, int *method, int *rows, int *stages);
/* Every wait of the staged step's copy pipeline (an mbarrier poll loop) is
 * bounded: after `polls` unsuccessful polls the waiting warp records
 * RR_ERR_WATCHDOG (reported by the next rr_sync, "a wait of the staged step's
 * pipeline timed out"), its CTA stops, and the CTA's copy-issuing thread waits
 * for the copies it has in flight before it exits.  polls < 0 restores the
 * default (2^24); 0 makes every wait give up at once, so the timeout path can
 * be exercised.  The state of a step whose wait gave up is not valid: set it
 * again (rr_init_state / rr_load).  No counterpart in the reference, whose
 * kernels do not wait on one another. */
rr_status rr_set_wait_limit(rr_solver *s, long long polls);
long long rr_get_wait_limit(const rr_solver *s);

#ifdef __cplusplus
}
#endif
#endif
