// rr_internal.h -- the solver object shared by the translation units of the
// library (rr_api.cu: single domains; rr_batch.cu: batches and the
// autotuner).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "rr_api.h"
#include "rr_dispatch.h"
#include "rr_kernels.cuh"

// The C library's rand() sequence after srand(seed) (the channel program's
// trip phases come from it), kept per solver: the additive-feedback generator
// r_i = r_{i-3} + r_{i-31} (mod 2^32), output r_i >> 1, seeded by
// r_0 = seed, r_i = 16807 r_{i-1} mod (2^31 - 1) for i < 31, r_i = r_{i-31}
// for 31 <= i < 34, the first 310 outputs discarded.
struct TripRand {
    int32_t r[34] = {};
    int k = 0;
    void seed(unsigned s0) {
        int32_t t[344];
        t[0] = (int32_t)s0;
        for (int i = 1; i < 31; i++) {
            long long w = (16807LL * (long long)t[i - 1]) % 2147483647LL;
            if (w < 0) w += 2147483647LL;
            t[i] = (int32_t)w;
        }
        for (int i = 31; i < 34; i++) t[i] = t[i - 31];
        for (int i = 34; i < 344; i++) t[i] = (int32_t)((uint32_t)t[i - 31] + (uint32_t)t[i - 3]);
        for (int i = 0; i < 34; i++) r[i] = t[310 + i];
        k = 0;
    }
    int next() {
        const int32_t v = (int32_t)((uint32_t)r[(k + 3) % 34] + (uint32_t)r[(k + 31) % 34]);
        r[k] = v;
        k = (k + 1) % 34;
        return (int)((uint32_t)v >> 1);
    }
};

struct rr_solver {
    rr_params p;
    const rr::Ops *ops = nullptr;
    rr::Geom g{};
    cudaStream_t stream = nullptr; // where the solver's work goes (the batch's stream while a member)
    cudaStream_t home = nullptr;   // the solver's own stream
    rr_batch *batch = nullptr;     // batch the solver is a member of
    void *buf[2] = {nullptr, nullptr};
    int cur = 0; // buffer holding the latest post-collision state
    long long istep = 0;
    bool ready = false;
    bool stepped = false; // a step ran since the state was set: the previous buffer is valid
    int *status = nullptr;   // device watchdog word
    int *pos = nullptr;      // device: internal population -> API population
    double *aux = nullptr;   // device FP64: rho, ux, uy, uz, taut (5 N)
    double *stat = nullptr;  // device FP64: diag partials + outputs + profile + accumulators
    long long acc_samples = 0;
    size_t bytes = 0;
    rr::LesTile tile{32, 8, 16};    // fused WALE step: x-y tile and z chunk
    int les_method = RR_LES_FUSED; // WALE step: fused z-marching tiles or two tile passes
    void *ubuf = nullptr;          // two-pass WALE step: velocity field (3 arrays of g.stride)
    rr::StepRange all{};      // every node, for grids with nx < 3 (general step)
    uint32_t *all_list = nullptr;
    uint32_t *edge_list = nullptr; // x-end nodes of rows on a y/z wall (tile step)
    uint32_t nedges = 0;
    int block = 256;
    int rows_group = 32; // tile step: rows per work-item group (autotuned)
    int dns_method = RR_DNS_TILE; // DNS step: tile step or staged step
    int stage_rows = 2, stages = 3; // staged step: rows per block, pipeline stages
    uint32_t stage_wait = rr::STAGE_WAIT_LIMIT; // staged step: polls before a pipeline wait gives up
    uint32_t *frow_list = nullptr;  // staged step: rows on a y or z face
    uint32_t nfrows = 0;
    cudaStream_t side = nullptr;     // staged step: the face-row launch, beside the interior one
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t copied = nullptr;    // rr_init_state from host buffers: the copies are done
    double *ffield = nullptr;        // trip forcing: the force fields of two steps (2 x 3 arrays of g.stride)
    TripRand trip_rng;
    double trip_phase = 0.0;
    uint32_t fdbc = 0;               // finite-difference wall closure: bit 0 y-lo, bit 1 y-hi
    // WALE with FDBC: tau_t of the wall nodes (2 nz nx each) of the collision
    // that wrote buf[b] in slot b (swapped with the buffers)
    double *fdbc_wt[2] = {nullptr, nullptr};
    double *fdbc_wt_mem = nullptr;
    cudaGraphExec_t graph = nullptr;
};

// sets this thread's rr_last_error() text and returns st
rr_status rr_internal_error(rr_status st, const char *fmt, ...);

namespace rr {

bool has_force(const rr_params &p);
// the step kind of a solver: the tile step (one launch, batchable) or not
inline bool tile_step(const rr_solver *s) { return !s->p.use_les && s->p.lx >= 3 && !s->g.bgk; }
// a tile-step solver the persistent batch kernel can step (its whole step is
// the one tile launch: no finite-difference closure pass after it)
inline bool batchable(const rr_solver *s) { return tile_step(s) && !s->fdbc; }
// the staged step applies: DNS, at least 3 nodes on every axis, rows a
// multiple of 16 bytes (bulk copies)
inline bool staged_ok(const rr_params &p, size_t elem) {
    return !p.use_les && p.collision == RR_COLL_RR && p.lx >= 3 && p.ly >= 3 && p.lz >= 3 &&
           ((size_t)p.lx * elem) % 16 == 0;
}
// one step of s from fin to fout on stream st (state bookkeeping is the
// caller's); i: the steps done before it (the trip forcing's step number), -1
// outside the trip phase
rr_status launch_one(rr_solver *s, const void *fin, void *fout, cudaStream_t st, long long i = -1);
// the force-field slot of step n (trip forcing)
double *trip_slot(rr_solver *s, long long n);
// the force of step n into its slot (redrawing the trip phase when due)
rr_status trip_prepare(rr_solver *s, long long n, cudaStream_t st);
// the solver is in its trip-forcing phase for the launch after i steps
inline bool trip_phase(const rr_solver *s, long long i) {
    return s->ffield && i >= 0 && i + 1 < s->p.trip_steps;
}
// drop the solver's captured step graph (launch shapes or buffers changed)
void drop_graph(rr_solver *s);
// tuned launch shapes of a size class, when the autotuner has seen it
bool tuned_rows_group(const rr_params &p, int *rows_group);
bool tuned_les_tile(const rr_params &p, LesTile *tile);
bool tuned_stage(const rr_params &p, int *method, int *rows, int *stages);
// detach s from its batch (the batch's work on s is finished first)
rr_status batch_detach(rr_solver *s);

} // namespace rr
