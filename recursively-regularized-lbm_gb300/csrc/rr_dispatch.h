// rr_dispatch.h -- host-side launch table, one per population storage type.
// Each rr_inst_<type>.cu instantiates the kernels of rr_kernels.cuh for its
// storage type and fills one Ops table; rr_api.cu picks the table at
// rr_create time.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace rr {

struct Geom;

// polls of an mbarrier before a wait of the staged step gives up (its
// default; rr_set_wait_limit changes the run-time limit of a solver)
constexpr uint32_t STAGE_WAIT_LIMIT = 1u << 24;

// bits of a solver's device watchdog word
constexpr int WATCH_DENSITY = 1; // density left (0.1, 10) or became NaN
constexpr int WATCH_STAGE_WAIT = 4; // a wait of the staged step's pipeline gave up

struct LesTile {
    int tx, ty, zchunk; // tile of the WALE step kernel (autotuned per size class)
};

// nodes covered by a list-driven step launch
struct StepRange {
    uint32_t count;
    const uint32_t *list;
};

// one launch of the finite-difference wall closure (rr_fdbc.cuh) over the
// FDBC y faces: after the step kernels, from the same input buffer
struct FdbcCall {
    int q;
    bool force;
    int mode;                 // 0 DNS step, 1 / 2 the WALE passes, 3 readout
    const void *fin;
    void *fout;
    const Geom *g;
    double om1, tau, cw;
    const double *F;          // uniform force (3)
    int *status;
    const double *ffp, *ffc;  // per-node forces (trip forcing) or NULL
    void *ubuf;               // WALE velocity field
    double *wt;               // WALE tau_t of the wall nodes, 2 nz nx (NULL for DNS): of fin's collision
    double *wt_out;           // ... and of this step's collision (mode 2)
    double *fo;               // readout: populations (or NULL) ...
    unsigned long long fo_stride;
    const int *pos;
    double *rho, *ux, *uy, *uz; // ... and moments (or NULL)
    uint32_t faces;           // bit 0: y-lo is FDBC, bit 1: y-hi
};

struct Ops {
    size_t elem_bytes;
    // one fused time step over the nodes of `r`: fin -> fout
    cudaError_t (*step)(int q, bool force, const void *fin, void *fout, const Geom &g, double om1,
                        const double F[3], int *status, const StepRange &r, int block,
                        cudaStream_t st);
    // one fused time step over the whole grid in one launch (needs nx >= 3);
    // edges: the x-end nodes of rows on a y/z wall face
    // rows_group: rows per work-item group (a multiple of 32)
    // ffp, ffc: per-node force fields of the streaming half and of the
    // collision (3 arrays of g.stride each; NULL: the uniform F; D3Q27 only)
    cudaError_t (*tile)(int q, bool force, const void *fin, void *fout, const Geom &g, double om1,
                        const double F[3], int *status, const uint32_t *edges, uint32_t nedges,
                        int rows_group, const double *ffp, const double *ffc, cudaStream_t st);
    // the staged step (needs nx * element size a multiple of 16): rows on a
    // y/z face (frows) in one launch, the interior rows in blocks of R rows
    // through an NS-stage shared-memory pipeline of bulk copies
    // (side, fork, join: a second stream and two events for the face-row
    // launch; side == NULL runs both launches on st); wait_limit: polls
    // before a pipeline wait gives up (the drain before a CTA exits always
    // takes STAGE_WAIT_LIMIT)
    cudaError_t (*staged)(int q, bool force, const void *fin, void *fout, const Geom &g, double om1,
                          const double F[3], int *status, const uint32_t *frows, uint32_t nfrows, int R, int NS,
                          uint32_t wait_limit, cudaStream_t st, cudaStream_t side, cudaEvent_t fork,
                          cudaEvent_t join);
    // the tile step's descriptor of one domain (TileArgs, written to out when
    // out != NULL) for a batch launch; returns its size, *nitems its warp items
    size_t (*tile_desc)(int q, const void *fin, void *fout, const Geom &g, double om1, const double F[3],
                        int *status, const uint32_t *edges, uint32_t nedges, int rows_group, void *out,
                        uint32_t *nitems);
    // one step of every domain of a batch: a persistent launch of `grid` CTAs
    // of `block` threads over the domains' CTAs (cta_begin: [ndom + 1] prefix
    // sums of ceil(32 nitems / block); cta_dom: domain of each CTA); desc:
    // device array of descriptors; chunked: contiguous walk instead of strided
    cudaError_t (*batch)(int q, bool force, const void *desc, const uint32_t *cta_begin, const uint32_t *cta_dom,
                         uint32_t ndom, uint32_t total_ctas, int block, int grid, int chunked, cudaStream_t st);
    // resident CTAs per SM of the batch kernel (0 on error)
    int (*batch_occupancy)(int q, bool force, int block);
    // fused time step with the WALE eddy viscosity
    cudaError_t (*step_les)(int q, bool force, const void *fin, void *fout, const Geom &g,
                            double tau, double cw, const double F[3], int *status,
                            const LesTile &tile, cudaStream_t st);
    // the same step in two tile launches (needs nx >= 3): velocities into ubuf
    // (3 arrays of g.stride in the compute type), then tau_t + collision;
    // pass 1 or 2 launches that pass alone, 0 both
    cudaError_t (*les2)(int q, bool force, const void *fin, void *fout, const Geom &g, double tau, double cw,
                        const double F[3], int *status, const uint32_t *edges, uint32_t nedges, int rows_group,
                        void *ubuf, const double *ffp, const double *ffc, int pass, cudaStream_t st);
    // post-stream populations / macroscopic fields from the post-collision buffer
    cudaError_t (*readout)(int q, bool force, const void *fin, const Geom &g, const double F[3],
                           double *fo, unsigned long long fo_stride, const int *pos, double *rho,
                           double *ux, double *uy, double *uz, const double *ff, cudaStream_t st);
    // state upload + first collision with given macros
    cudaError_t (*upload)(int q, bool force, void *fout, const Geom &g, double tau,
                          const double F[3], const double *fi, unsigned long long fi_stride,
                          const int *pos, const double *rho, const double *ux, const double *uy,
                          const double *uz, const double *taut, const double *ff, cudaStream_t st);
    // the finite-difference wall closure of the FDBC faces
    cudaError_t (*fdbc)(const FdbcCall &c, cudaStream_t st);
};

const Ops &ops_f64();
const Ops &ops_f32();
const Ops &ops_f16();
const Ops &ops_bf16();

// FP64 helpers shared by all storage types (rr_aux.cu)
cudaError_t launch_wale(const Geom &g, double cw, const double *ux, const double *uy,
                        const double *uz, double *taut, cudaStream_t st);

} // namespace rr
