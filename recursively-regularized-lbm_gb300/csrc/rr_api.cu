// rr_api.cu -- host side of the C ABI declared in include/rr_api.h.
//
// A solver owns two population buffers (ping-pong), a CUDA stream, a watchdog
// word and, lazily, FP64 scratch for readouts and statistics.  rr_step()
// enqueues fused step kernels (CUDA graphs of GRAPH_STEPS steps for long
// runs); nothing synchronises until a readout or rr_sync().
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "rr_api.h"
#include "rr_aux.h"
#include "rr_dispatch.h"
#include "rr_internal.h"
#include "rr_kernels.cuh"

namespace {

thread_local std::string g_err;

rr_status fail(rr_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

#define RR_CK(call)                                                                            \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(RR_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                   \
    } while (0)

constexpr int GRAPH_STEPS = 32; // steps per captured graph (even: ends on the same buffer)

const rr::Ops &ops_for(int storage) {
    switch (storage) {
    case RR_STORE_F64: return rr::ops_f64();
    case RR_STORE_F32: return rr::ops_f32();
    case RR_STORE_F16: return rr::ops_f16();
    default: return rr::ops_bf16();
    }
}

unsigned long long padded_stride(uint32_t n) { return ((unsigned long long)n + 63ull) & ~63ull; }

// velocity field of the two-pass WALE step (compute type: FP64 for FP64 storage)
size_t les_ubuf_bytes(const rr_params &p) {
    if (!p.use_les || p.lx < 3) return 0;
    const uint32_t n = (uint32_t)p.lx * p.ly * p.lz;
    return 3 * padded_stride(n) * (p.storage == RR_STORE_F64 ? sizeof(double) : sizeof(float));
}


rr_status validate(const rr_params *p) {
    if (!p) return fail(RR_ERR_INVALID, "params is NULL");
    if (p->lx < 1 || p->ly < 1 || p->lz < 1)
        return fail(RR_ERR_INVALID, "grid %dx%dx%d must be positive", p->lx, p->ly, p->lz);
    const double n = (double)p->lx * p->ly * p->lz;
    if (n > 2147483647.0) return fail(RR_ERR_INVALID, "grid has %.0f nodes, limit 2^31-1", n);
    if (p->q != 19 && p->q != 27) return fail(RR_ERR_INVALID, "q = %d, must be 19 or 27", p->q);
    if (p->storage < RR_STORE_F64 || p->storage > RR_STORE_BF16)
        return fail(RR_ERR_INVALID, "storage = %d unknown", p->storage);
    if (!(p->tau > 0.5)) return fail(RR_ERR_INVALID, "tau = %g must exceed 0.5", p->tau);
    if (p->order != RR_ORDER_CUDA && p->order != RR_ORDER_FORTRAN)
        return fail(RR_ERR_INVALID, "order = %d unknown", p->order);
    if (p->q == 19 && p->order != RR_ORDER_FORTRAN)
        return fail(RR_ERR_INVALID, "D3Q19 populations exist only in the Fortran ordering");
    const int n3[3] = {p->lx, p->ly, p->lz};
    for (int f = 0; f < 6; f++) {
        if (p->face[f] < RR_FACE_PERIODIC || p->face[f] > RR_FACE_FDBC)
            return fail(RR_ERR_INVALID, "face[%d] = %d unknown", f, p->face[f]);
        if (p->face[f] != RR_FACE_PERIODIC && n3[f / 2] < 2)
            return fail(RR_ERR_INVALID, "a wall on face %d needs at least 2 nodes across", f);
        if (p->face[f] == RR_FACE_PERIODIC &&
            (p->uwall[f][0] != 0.0 || p->uwall[f][1] != 0.0 || p->uwall[f][2] != 0.0))
            return fail(RR_ERR_INVALID, "face %d is periodic but has a wall velocity", f);
    }
    if ((p->face[0] == RR_FACE_PERIODIC) != (p->face[1] == RR_FACE_PERIODIC) ||
        (p->face[2] == RR_FACE_PERIODIC) != (p->face[3] == RR_FACE_PERIODIC) ||
        (p->face[4] == RR_FACE_PERIODIC) != (p->face[5] == RR_FACE_PERIODIC))
        return fail(RR_ERR_INVALID, "an axis must be periodic on both faces or on neither");
    if (p->use_les && !(p->cw >= 0.0)) return fail(RR_ERR_INVALID, "cw = %g", p->cw);
    if (p->rounding != RR_ROUND_NEAREST && p->rounding != RR_ROUND_STOCHASTIC)
        return fail(RR_ERR_INVALID, "rounding = %d unknown", p->rounding);
    if (p->trip_steps < 0) return fail(RR_ERR_INVALID, "trip_steps = %d", p->trip_steps);
    if (p->trip_steps > 0 && (p->q != 27 || p->lx < 3))
        return fail(RR_ERR_UNSUPPORTED, "trip forcing needs D3Q27 and lx >= 3");
    // forcing_GP scales its field by force_in_x (macrovar.cu:76-115)
    if (p->trip_steps > 0 && p->force[0] == 0.0)
        return fail(RR_ERR_UNSUPPORTED, "trip forcing needs a body force along x (force[0] != 0)");
    if (p->collision != RR_COLL_RR && p->collision != RR_COLL_BGK)
        return fail(RR_ERR_INVALID, "collision = %d unknown", p->collision);
    const bool fdbc = p->face[2] == RR_FACE_FDBC || p->face[3] == RR_FACE_FDBC;
    for (int f : {0, 1, 4, 5})
        if (p->face[f] == RR_FACE_FDBC)
            return fail(RR_ERR_UNSUPPORTED, "the finite-difference closure is for the y faces only (face %d)", f);
    if (fdbc) {
        // BC.cu:129-309: x and z periodic, walls at rest, rows 1 and 2 inside
        if (p->face[0] != RR_FACE_PERIODIC || p->face[4] != RR_FACE_PERIODIC)
            return fail(RR_ERR_UNSUPPORTED, "the finite-difference closure needs periodic x and z");
        for (int f = 2; f < 4; f++)
            if (p->face[f] == RR_FACE_FDBC && (p->uwall[f][0] != 0.0 || p->uwall[f][1] != 0.0 || p->uwall[f][2] != 0.0))
                return fail(RR_ERR_UNSUPPORTED, "the finite-difference closure takes walls at rest (face %d)", f);
        if (p->ly < 4) return fail(RR_ERR_UNSUPPORTED, "the finite-difference closure needs ly >= 4");
        if (p->collision != RR_COLL_RR)
            return fail(RR_ERR_UNSUPPORTED, "the finite-difference closure needs the RR collision");
        if (p->use_les && p->lx < 3)
            return fail(RR_ERR_UNSUPPORTED, "WALE with the finite-difference closure needs lx >= 3");
    }
    if (p->collision == RR_COLL_BGK) {
        if (p->q != 27 || p->use_les || p->lx < 3 || p->trip_steps > 0)
            return fail(RR_ERR_UNSUPPORTED, "the BGK collision needs D3Q27, DNS, lx >= 3 and no trip forcing");
        for (int f = 0; f < 6; f++)
            if (p->face[f] == RR_FACE_WALL)
                return fail(RR_ERR_UNSUPPORTED, "the BGK collision takes bounce-back walls (RR_FACE_WALL_BB), "
                                                "not the regularized closure");
    }
    return RR_OK;
}

} // namespace

namespace {

std::vector<int> api_positions(const rr_params &p) {
    // internal order: CUDA order for D3Q27, Fortran (= only) order for D3Q19
    std::vector<int> pos(p.q);
    for (int i = 0; i < p.q; i++) pos[i] = i;
    if (p.q == 27 && p.order == RR_ORDER_FORTRAN)
        for (int j = 0; j < 27; j++) pos[rr::FORTRAN_TO_CUDA_27[j]] = j;
    return pos;
}

size_t stat_doubles(const rr_params &p) {
    // diag partials, 4 outputs, profile (12 ly), accumulators (12 ly)
    return 4 * (size_t)rr::DIAG_MAX_BLOCKS + 4 + 24 * (size_t)p.ly;
}

rr_status ensure_aux(rr_solver *s) {
    if (s->aux) return RR_OK;
    const size_t n = s->g.n;
    if (cudaMallocAsync(&s->aux, 5 * n * sizeof(double), s->stream) != cudaSuccess) {
        s->aux = nullptr;
        cudaGetLastError();
        return fail(RR_ERR_NOMEM, "cannot allocate %zu bytes of readout scratch", 5 * n * sizeof(double));
    }
    s->bytes += 5 * n * sizeof(double);
    return RR_OK;
}

rr_status set_device(const rr_solver *s) {
    RR_CK(cudaSetDevice(s->p.device));
    return RR_OK;
}

// the force field of the state a readout shows (step istep), while the trip
// forcing has made it a field
const double *readout_field(rr_solver *s) {
    return (s->ffield && s->istep >= 1 && s->istep < s->p.trip_steps) ? rr::trip_slot(s, s->istep) : nullptr;
}

// the readout of the state after the last step from the previous buffer:
// populations (fo, reference layout) and/or moments; the wall rows of the
// finite-difference closure's faces come from its own kernel
cudaError_t readout_state(rr_solver *s, double *fo, double *rho, double *ux, double *uy, double *uz) {
    const void *fin = s->buf[1 - s->cur];
    const double *ff = readout_field(s);
    cudaError_t e = s->ops->readout(s->p.q, rr::has_force(s->p), fin, s->g, s->p.force, fo, s->g.n, s->pos, rho, ux,
                                    uy, uz, ff, s->stream);
    if (e != cudaSuccess || !s->fdbc) return e;
    rr::FdbcCall fc{};
    fc.q = s->p.q;
    fc.force = rr::has_force(s->p);
    fc.mode = 3;
    fc.fin = fin;
    fc.g = &s->g;
    fc.tau = s->p.tau;
    fc.F = s->p.force;
    fc.status = s->status;
    fc.ffp = ff;
    fc.ffc = ff; // (no collision in a readout)
    fc.wt = s->fdbc_wt[1 - s->cur];
    fc.fo = fo;
    fc.fo_stride = s->g.n;
    fc.pos = s->pos;
    fc.rho = rho;
    fc.ux = ux;
    fc.uy = uy;
    fc.uz = uz;
    fc.faces = s->fdbc;
    return s->ops->fdbc(fc, s->stream);
}

// rho, u (and taut) of the current state into aux
rr_status readout_macros(rr_solver *s, bool want_taut) {
    rr_status st = ensure_aux(s);
    if (st != RR_OK) return st;
    const size_t n = s->g.n;
    double *rho = s->aux, *ux = rho + n, *uy = ux + n, *uz = uy + n, *tt = uz + n;
    // the previous buffer holds the post-collision state the last step read
    RR_CK(readout_state(s, nullptr, rho, ux, uy, uz));
    if (want_taut) RR_CK(rr::launch_wale(s->g, s->p.cw, ux, uy, uz, tt, s->stream));
    return RR_OK;
}

rr_status copy_out(rr_solver *s, double *dst, const double *src, size_t count, int where) {
    if (!dst) return RR_OK;
    RR_CK(cudaMemcpyAsync(dst, src, count * sizeof(double),
                          where == RR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          s->stream));
    return RR_OK;
}

rr_status launch_steps(rr_solver *s, int n) {
    for (int k = 0; k < n; k++) {
        rr_status st = rr::launch_one(s, s->buf[s->cur], s->buf[1 - s->cur], s->stream, s->istep + k);
        if (st != RR_OK) return st;
        s->cur = 1 - s->cur;
    }
    return RR_OK;
}

rr_status build_graph(rr_solver *s) {
    if (s->graph) return RR_OK;
    // captured from buffer 0; GRAPH_STEPS is even, so it ends on buffer 0
    const int saved = s->cur;
    s->cur = 0;
    cudaGraph_t graph;
    RR_CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    rr_status st = launch_steps(s, GRAPH_STEPS);
    cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
    s->cur = saved;
    if (st != RR_OK) return st;
    if (e != cudaSuccess) return fail(RR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        s->graph = nullptr;
        return fail(RR_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    }
    return RR_OK;
}

rr_status write_file(const std::string &path, const void *data, size_t bytes, const char *mode) {
    FILE *fp = fopen(path.c_str(), mode);
    if (!fp) return fail(RR_ERR_IO, "cannot open %s: %s", path.c_str(), strerror(errno));
    size_t w = fwrite(data, 1, bytes, fp);
    int e = fflush(fp);
    fclose(fp);
    if (w != bytes || e != 0) return fail(RR_ERR_IO, "short write to %s", path.c_str());
    return RR_OK;
}

rr_status ensure_dir(const char *dir) {
    struct stat sb;
    if (stat(dir, &sb) == 0) return RR_OK;
    if (mkdir(dir, 0700) != 0 && errno != EEXIST) return fail(RR_ERR_IO, "cannot create %s", dir);
    return RR_OK;
}

} // namespace

namespace rr {

bool has_force(const rr_params &p) { return p.force[0] != 0.0 || p.force[1] != 0.0 || p.force[2] != 0.0; }

// the force-field slot of step n
double *trip_slot(rr_solver *s, long long n) { return s->ffield + (size_t)(n & 1) * 3 * s->g.stride; }

// the force of step n into its slot: the trip field while n < trip_steps
// (redrawing the phase every 2000 steps), the uniform force after
rr_status trip_prepare(rr_solver *s, long long n, cudaStream_t st) {
    const int trip = n < s->p.trip_steps ? 1 : 0;
    double amp = 0.0;
    if (trip) {
        if (n % 2000 == 0) s->trip_phase = (double)s->trip_rng.next() / 2147483647.0;
        amp = (100.0 * 3.0 / s->p.ly) * sin(2 * acos(-1.0) * (double)n / 2000.0);
    }
    RR_CK(rr::launch_trip_force(trip_slot(s, n), s->g.stride, s->p.lx, s->p.ly, s->p.lz, trip, amp,
                                s->trip_phase, s->p.force, st));
    return RR_OK;
}

rr_status launch_one(rr_solver *s, const void *fin, void *fout, cudaStream_t st, long long i) {
    const bool force = rr::has_force(s->p);
    // in the trip phase: the force of step i+1 (walls and moments) and of
    // step i+2 (the collision), per node
    const double *ffp = nullptr, *ffc = nullptr;
    if (trip_phase(s, i)) {
        rr_status ts = trip_prepare(s, i + 2, st);
        if (ts != RR_OK) return ts;
        ffp = trip_slot(s, i + 1);
        ffc = trip_slot(s, i + 2);
    }
    rr::FdbcCall fc{};
    if (s->fdbc) {
        fc.q = s->p.q;
        fc.force = force;
        fc.fin = fin;
        fc.fout = fout;
        fc.g = &s->g;
        fc.om1 = 1.0 - 1.0 / s->p.tau;
        fc.tau = s->p.tau;
        fc.cw = s->p.cw;
        fc.F = s->p.force;
        fc.status = s->status;
        fc.ffp = ffp;
        fc.ffc = ffc;
        fc.ubuf = s->ubuf;
        const int in = fin == s->buf[1] ? 1 : 0;
        fc.wt = s->fdbc_wt[in];
        fc.wt_out = s->fdbc_wt[1 - in];
        fc.faces = s->fdbc;
    }
    // the closure's kernel beside a tile launch, which leaves the closure's
    // rows alone: on the side stream, launched first so that its CTAs are
    // resident before the tile step fills the SMs
    auto beside = [&](int mode, auto &&main) -> rr_status {
        fc.mode = mode;
        RR_CK(cudaEventRecord(s->fork, st));
        RR_CK(cudaStreamWaitEvent(s->side, s->fork, 0));
        // once the side stream is forked, every path joins it again before
        // returning (a capture must not end with the fork open)
        const cudaError_t ef = s->ops->fdbc(fc, s->side);
        const rr_status r = ef == cudaSuccess ? main() : RR_OK;
        cudaError_t e = cudaEventRecord(s->join, s->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, s->join, 0);
        if (ef != cudaSuccess)
            return fail(RR_ERR_CUDA, "finite-difference closure launch failed: %s", cudaGetErrorString(ef));
        if (r != RR_OK) return r;
        if (e != cudaSuccess) return fail(RR_ERR_CUDA, "side-stream join failed: %s", cudaGetErrorString(e));
        return RR_OK;
    };
    if (s->p.use_les) {
        if (s->fdbc) {
            // the wall rows' velocities are the closure's before tau_t reads them
            for (int pass = 1; pass <= 2; pass++) {
                rr_status r = beside(pass, [&]() -> rr_status {
                    RR_CK(s->ops->les2(s->p.q, force, fin, fout, s->g, s->p.tau, s->p.cw, s->p.force, s->status,
                                       s->edge_list, s->nedges, s->rows_group, s->ubuf, ffp, ffc, pass, st));
                    return RR_OK;
                });
                if (r != RR_OK) return r;
            }
            return RR_OK;
        }
        if ((s->les_method == RR_LES_TWO_PASS || ffp) && s->ubuf)
            RR_CK(s->ops->les2(s->p.q, force, fin, fout, s->g, s->p.tau, s->p.cw, s->p.force, s->status,
                               s->edge_list, s->nedges, s->rows_group, s->ubuf, ffp, ffc, 0, st));
        else
            RR_CK(s->ops->step_les(s->p.q, force, fin, fout, s->g, s->p.tau, s->p.cw, s->p.force, s->status,
                                   s->tile, st));
    } else if (s->p.lx >= 3 && s->dns_method == RR_DNS_STAGED && s->frow_list && !ffp && !s->g.bgk) {
        RR_CK(s->ops->staged(s->p.q, force, fin, fout, s->g, 1.0 - 1.0 / s->p.tau, s->p.force, s->status,
                             s->frow_list, s->nfrows, s->stage_rows, s->stages, s->stage_wait, st, s->side, s->fork,
                             s->join));
    } else if (s->p.lx >= 3) {
        auto tile = [&]() -> rr_status {
            RR_CK(s->ops->tile(s->p.q, force, fin, fout, s->g, 1.0 - 1.0 / s->p.tau, s->p.force, s->status,
                               s->edge_list, s->nedges, s->rows_group, ffp, ffc, st));
            return RR_OK;
        };
        return s->fdbc ? beside(0, tile) : tile();
    } else {
        RR_CK(s->ops->step(s->p.q, force, fin, fout, s->g, 1.0 - 1.0 / s->p.tau, s->p.force, s->status, s->all,
                           s->block, st));
    }
    // the staged and the thin-grid steps write the closure's rows: it runs after them
    if (s->fdbc) {
        fc.mode = 0;
        RR_CK(s->ops->fdbc(fc, st));
    }
    return RR_OK;
}

void drop_graph(rr_solver *s) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
}

} // namespace rr

// sets this thread's rr_last_error() text for entry points in other files
rr_status rr_internal_error(rr_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

extern "C" {

const char *rr_last_error(void) { return g_err.c_str(); }

rr_status rr_params_default(rr_params *p) {
    if (!p) return fail(RR_ERR_INVALID, "params is NULL");
    memset(p, 0, sizeof(*p));
    // parameters.h:9-11 and globals.cu:33-38
    p->lx = p->ly = p->lz = 64;
    p->q = 27;
    p->use_les = 0;
    const double Re = 180.0, visc = 0.000622;
    const double u0 = 2.0 * Re * visc / p->ly;
    p->tau = 3.0 * visc + 0.5;
    p->cw = 0.5;
    p->force[0] = 2.0 * u0 * u0 / p->ly;
    p->face[2] = p->face[3] = RR_FACE_WALL;
    p->storage = RR_STORE_F64;
    p->order = RR_ORDER_CUDA;
    p->device = 0;
    p->ustar = u0;
    p->ystar = visc / u0;
    p->rounding = RR_ROUND_STOCHASTIC;
    return RR_OK;
}

size_t rr_bytes_for(const rr_params *p) {
    if (!p || validate(p) != RR_OK) return 0;
    const uint32_t n = (uint32_t)p->lx * p->ly * p->lz;
    const size_t elem = p->storage == RR_STORE_F64 ? 8 : p->storage == RR_STORE_F32 ? 4 : 2;
    size_t b = 2 * (size_t)p->q * padded_stride(n) * elem + 256 + stat_doubles(*p) * sizeof(double);
    b += les_ubuf_bytes(*p);
    // edge-node list of the tile step (x-ends of the rows on a y/z wall face)
    // and face-row list of the staged step
    if (p->lx >= 3) b += 2 * sizeof(uint32_t) * (size_t)(2 * p->lz + 2 * p->ly);
    if (rr::staged_ok(*p, elem)) b += sizeof(uint32_t) * (size_t)(2 * p->lz + 2 * p->ly);
    if (p->trip_steps > 0) b += 6 * padded_stride(n) * sizeof(double);
    // wall tau_t of WALE with the finite-difference closure: two slots
    if (p->use_les && (p->face[2] == RR_FACE_FDBC || p->face[3] == RR_FACE_FDBC))
        b += 4 * (size_t)p->lx * p->lz * sizeof(double);
    return b;
}

rr_status rr_create(const rr_params *p, rr_solver **out) {
    if (!out) return fail(RR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    rr_status st = validate(p);
    if (st != RR_OK) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(RR_ERR_CUDA, "no CUDA device");
    }
    if (p->device < 0 || p->device >= ndev) return fail(RR_ERR_INVALID, "device %d of %d", p->device, ndev);
    rr_solver *s = new rr_solver();
    s->p = *p;
    s->ops = &ops_for(p->storage);
    rr::Geom &g = s->g;
    g.nx = p->lx;
    g.ny = p->ly;
    g.nz = p->lz;
    g.n = (uint32_t)p->lx * p->ly * p->lz;
    g.stride = padded_stride(g.n);
    g.wallmask = 0;
    for (int f = 0; f < 6; f++) {
        g.face[f] = p->face[f];
        if (p->face[f] != RR_FACE_PERIODIC) g.wallmask |= 1u << f;
        for (int a = 0; a < 3; a++) g.uw[f][a] = p->uwall[f][a];
    }
    auto cleanup = [&](rr_status code) {
        rr_destroy(s);
        return code;
    };
    if (set_device(s) != RR_OK) return cleanup(RR_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(fail(RR_ERR_CUDA, "stream creation failed"));
    s->home = s->stream;
    const size_t bytes = (size_t)p->q * g.stride * s->ops->elem_bytes;
    for (int b = 0; b < 2; b++) {
        if (cudaMallocAsync(&s->buf[b], bytes, s->stream) != cudaSuccess) {
            cudaGetLastError();
            s->buf[b] = nullptr;
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate %zu bytes of populations", bytes));
        }
        s->bytes += bytes;
    }
    // one 256-byte block: the watchdog word, then the 27-entry population order
    if (cudaMallocAsync(&s->status, 256, s->stream) != cudaSuccess || cudaMemsetAsync(s->status, 0, 256, s->stream) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(fail(RR_ERR_NOMEM, "cannot allocate the watchdog word"));
    }
    s->pos = s->status + 4;
    std::vector<int> pos = api_positions(*p);
    if (cudaMemcpyAsync(s->pos, pos.data(), pos.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        return cleanup(fail(RR_ERR_CUDA, "cannot upload the population order"));
    const size_t sd = stat_doubles(*p) * sizeof(double);
    if (cudaMallocAsync(&s->stat, sd, s->stream) != cudaSuccess || cudaMemsetAsync(s->stat, 0, sd, s->stream) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(fail(RR_ERR_NOMEM, "cannot allocate statistics buffers"));
    }
    s->bytes += 256 + sd;
    // the tile step's edge nodes: x = 0 and x = nx-1 of every row lying on a
    // y or z wall face
    if (p->lx >= 3) {
        std::vector<uint32_t> edges;
        for (int z = 0; z < p->lz; z++)
            for (int y = 0; y < p->ly; y++) {
                const bool yzw = (p->face[2] != RR_FACE_PERIODIC && y == 0) ||
                                 (p->face[3] != RR_FACE_PERIODIC && y == p->ly - 1) ||
                                 (p->face[4] != RR_FACE_PERIODIC && z == 0) ||
                                 (p->face[5] != RR_FACE_PERIODIC && z == p->lz - 1);
                if (!yzw) continue;
                const uint32_t row = (uint32_t)z * p->ly + y;
                edges.push_back(row * p->lx);
                edges.push_back(row * p->lx + p->lx - 1);
            }
        if (!edges.empty()) {
            const size_t lb = edges.size() * sizeof(uint32_t);
            if (cudaMallocAsync(&s->edge_list, lb, s->stream) != cudaSuccess) {
                cudaGetLastError();
                s->edge_list = nullptr;
                return cleanup(fail(RR_ERR_NOMEM, "cannot allocate the edge-node list"));
            }
            if (cudaMemcpyAsync(s->edge_list, edges.data(), lb, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
                return cleanup(fail(RR_ERR_CUDA, "cannot upload the edge-node list"));
            s->nedges = (uint32_t)edges.size();
            s->bytes += lb;
        }
    }
    // the staged step's face rows (rows with y or z on a face, any kind), and
    // its block shape: about 28 KB of populations per stage, two stages
    if ((rr::staged_ok(*p, s->ops->elem_bytes) || p->face[2] == RR_FACE_FDBC || p->face[3] == RR_FACE_FDBC) &&
        (cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming) != cudaSuccess))
        return cleanup(fail(RR_ERR_CUDA, "cannot create the side stream"));
    if (rr::staged_ok(*p, s->ops->elem_bytes)) {
        // grouped by the faces a row lies on (z-lo, z-hi, y-lo, y-hi, then the
        // edge rows), so that neighbouring warps run the same compiled face path
        std::vector<uint32_t> frows;
        std::vector<uint32_t> by_kind[5];
        for (int z = 0; z < p->lz; z++)
            for (int y = 0; y < p->ly; y++) {
                const bool yf = y == 0 || y == p->ly - 1, zf = z == 0 || z == p->lz - 1;
                if (!yf && !zf) continue;
                const int kind = (yf && zf) ? 4 : zf ? (z == 0 ? 0 : 1) : (y == 0 ? 2 : 3);
                by_kind[kind].push_back((uint32_t)z * p->ly + y);
            }
        for (auto &v : by_kind) frows.insert(frows.end(), v.begin(), v.end());
        const size_t lb = frows.size() * sizeof(uint32_t);
        if (cudaMallocAsync(&s->frow_list, lb, s->stream) != cudaSuccess) {
            cudaGetLastError();
            s->frow_list = nullptr;
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate the face-row list"));
        }
        if (cudaMemcpyAsync(s->frow_list, frows.data(), lb, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
            return cleanup(fail(RR_ERR_CUDA, "cannot upload the face-row list"));
        s->nfrows = (uint32_t)frows.size();
        s->bytes += lb;
        const size_t row_bytes = (size_t)p->q * p->lx * s->ops->elem_bytes;
        s->stage_rows = (int)std::max<size_t>(
            1, std::min<size_t>({(28672 + row_bytes / 2) / row_bytes, (size_t)p->ly - 2, 32}));
        s->stages = 2;
    }
    // grids thinner than 3 nodes in x run the list-driven general step over
    // every node; all others the one-launch tile step
    if (p->lx < 3) {
        std::vector<uint32_t> all(g.n);
        for (uint32_t i = 0; i < g.n; i++) all[i] = i;
        const size_t lb = all.size() * sizeof(uint32_t);
        if (cudaMallocAsync(&s->all_list, lb, s->stream) != cudaSuccess) {
            cudaGetLastError();
            s->all_list = nullptr;
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate the node list"));
        }
        if (cudaMemcpyAsync(s->all_list, all.data(), lb, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
            return cleanup(fail(RR_ERR_CUDA, "cannot upload the node list"));
        s->all.count = g.n;
        s->all.list = s->all_list;
        s->bytes += lb;
    }
    g.sround = (p->rounding == RR_ROUND_STOCHASTIC) ? 1 : 0;
    g.bgk = p->collision == RR_COLL_BGK ? 1 : 0;
    if (const size_t ub = les_ubuf_bytes(*p)) {
        if (cudaMallocAsync(&s->ubuf, ub, s->stream) != cudaSuccess) {
            cudaGetLastError();
            s->ubuf = nullptr;
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate %zu bytes of WALE velocity field", ub));
        }
        s->bytes += ub;
        s->les_method = RR_LES_TWO_PASS;
    } else {
        s->les_method = RR_LES_FUSED;
    }
    s->fdbc = (p->face[2] == RR_FACE_FDBC ? 1u : 0u) | (p->face[3] == RR_FACE_FDBC ? 2u : 0u);
    // the tile step leaves the closure's rows to fdbc_kernel (the staged and
    // thin-grid steps write them and the closure runs after them)
    g.fdbc = s->fdbc;
    if (s->fdbc && p->use_les) {
        const size_t slot = 2 * (size_t)p->lx * p->lz;
        if (cudaMallocAsync(&s->fdbc_wt_mem, 2 * slot * sizeof(double), s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->fdbc_wt_mem, 0, 2 * slot * sizeof(double), s->stream) != cudaSuccess) {
            cudaGetLastError();
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate %zu bytes of wall tau_t", 2 * slot * sizeof(double)));
        }
        s->fdbc_wt[0] = s->fdbc_wt_mem;
        s->fdbc_wt[1] = s->fdbc_wt_mem + slot;
        s->bytes += 2 * slot * sizeof(double);
    }
    if (p->trip_steps > 0) {
        const size_t fb = 6 * (size_t)g.stride * sizeof(double);
        if (cudaMallocAsync(&s->ffield, fb, s->stream) != cudaSuccess) {
            cudaGetLastError();
            s->ffield = nullptr;
            return cleanup(fail(RR_ERR_NOMEM, "cannot allocate %zu bytes of trip force fields", fb));
        }
        s->bytes += fb;
    }
    // LES tile by size class: full 32-wide rows when x allows, else 16
    s->tile.tx = p->lx >= 32 ? 32 : 16;
    s->tile.ty = 256 / s->tile.tx;
    s->tile.zchunk = p->lz >= 64 ? 16 : (p->lz >= 16 ? 8 : p->lz);
    // launch shapes the autotuner found for this size class, if any
    rr::tuned_les_tile(*p, &s->tile);
    if (s->frow_list) rr::tuned_stage(*p, &s->dns_method, &s->stage_rows, &s->stages);
    rr::tuned_rows_group(*p, &s->rows_group);
    // the allocations and uploads above are ordered on the solver's stream
    // (stream-ordered allocation: creating or destroying a solver never waits
    // for other solvers' work on the device); complete them here
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return cleanup(fail(RR_ERR_CUDA, "solver set-up failed: %s", cudaGetErrorString(cudaGetLastError())));
    *out = s;
    return RR_OK;
}

rr_status rr_destroy(rr_solver *s) {
    if (!s) return RR_OK;
    cudaSetDevice(s->p.device);
    if (s->batch) rr::batch_detach(s);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    // stream-ordered frees on the solver's own stream: no device-wide wait
    void *mem[] = {s->buf[0],  s->buf[1],   s->status,    s->aux,    s->stat,       s->all_list,
                   s->edge_list, s->ubuf, s->frow_list, s->ffield, s->fdbc_wt_mem};
    for (void *m : mem)
        if (m) {
            if (s->home) cudaFreeAsync(m, s->home);
            else cudaFree(m);
        }
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->copied) cudaEventDestroy(s->copied);
    if (s->join) cudaEventDestroy(s->join);
    if (s->home) cudaStreamDestroy(s->home);
    cudaGetLastError();
    delete s;
    return RR_OK;
}

namespace {

// the state upload of a run that starts after step istep0 (0, or a restart)
rr_status init_state_at(rr_solver *s, const double *f, const double *rho, const double *ux, const double *uy,
                        const double *uz, int where, long long istep0) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (!rho || !ux || !uy || !uz) return fail(RR_ERR_INVALID, "rho, ux, uy, uz are required");
    if (s->batch) return fail(RR_ERR_STATE, "the solver is a member of a batch: remove it to set its state");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    const size_t n = s->g.n;
    const size_t nf = f ? (size_t)s->p.q * n : 0;
    double *tmp = nullptr;
    const size_t tmp_count = 5 * n + nf;
    RR_CK(cudaMallocAsync(&tmp, tmp_count * sizeof(double), s->stream));
    double *d_rho = tmp, *d_ux = tmp + n, *d_uy = d_ux + n, *d_uz = d_uy + n, *d_tt = d_uz + n;
    double *d_f = f ? d_tt + n : nullptr;
    const cudaMemcpyKind kind = where == RR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e = cudaSuccess;
    const double *src[4] = {rho, ux, uy, uz};
    double *dst[4] = {d_rho, d_ux, d_uy, d_uz};
    for (int k = 0; k < 4 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), kind, s->stream);
    if (e == cudaSuccess && f) e = cudaMemcpyAsync(d_f, f, nf * sizeof(double), kind, s->stream);
    // host buffers: the call returns once they are copied (the upload runs on)
    if (e == cudaSuccess && where == RR_HOST) {
        if (!s->copied) e = cudaEventCreateWithFlags(&s->copied, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(s->copied, s->stream);
    }
    // the reference's first step computes tau_t from these macros (main.cu:375-379)
    if (e == cudaSuccess && s->p.use_les) e = rr::launch_wale(s->g, s->p.cw, d_ux, d_uy, d_uz, d_tt, s->stream);
    // the trip forcing restarts with the run: srand(12345), phase 0; the
    // first collision (step istep0 + 1) takes that step's force
    const double *ff = nullptr;
    if (e == cudaSuccess && s->ffield) {
        s->trip_rng.seed(12345);
        s->trip_phase = 0.0;
        if (istep0 + 1 < s->p.trip_steps) {
            rr_status ts = rr::trip_prepare(s, istep0 + 1, s->stream);
            if (ts != RR_OK) {
                cudaFreeAsync(tmp, s->stream);
                return ts;
            }
            ff = rr::trip_slot(s, istep0 + 1);
        }
    }
    if (e == cudaSuccess)
        e = s->ops->upload(s->p.q, rr::has_force(s->p), s->buf[0], s->g, s->p.tau, s->p.force, d_f, n,
                           s->pos, d_rho, d_ux, d_uy, d_uz, s->p.use_les ? d_tt : nullptr, ff, s->stream);
    // the finite-difference closure of step istep0 + 1 takes that step's tau_t
    // at the wall nodes: kept with the buffer the upload wrote
    if (e == cudaSuccess && s->fdbc_wt[0]) e = rr::launch_wall_rows(s->g, d_tt, s->fdbc_wt[0], s->stream);
    cudaError_t e2 = cudaFreeAsync(tmp, s->stream);
    if (e != cudaSuccess) return fail(RR_ERR_CUDA, "state upload failed: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(RR_ERR_CUDA, "cudaFreeAsync: %s", cudaGetErrorString(e2));
    // buffer 0 now holds the post-collision state of step 1; the first step's
    // "previous buffer" (its own input for readouts) is buffer 1, which gets the
    // same role after the first rr_step.  Until then readouts are of the input.
    s->cur = 0;
    s->istep = istep0;
    s->ready = true;
    s->stepped = false;
    RR_CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
    if (where == RR_HOST) RR_CK(cudaEventSynchronize(s->copied));
    return RR_OK;
}

} // namespace

rr_status rr_init_state(rr_solver *s, const double *f, const double *rho, const double *ux,
                        const double *uy, const double *uz, int where) {
    return init_state_at(s, f, rho, ux, uy, uz, where, 0);
}

rr_status rr_step(rr_solver *s, int nsteps) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (!s->ready) return fail(RR_ERR_STATE, "rr_step before rr_init_state / rr_load");
    if (nsteps < 0) return fail(RR_ERR_INVALID, "nsteps = %d", nsteps);
    if (s->batch) return fail(RR_ERR_STATE, "the solver is a member of a batch: step it with rr_batch_step");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    int left = nsteps;
    // steps of the trip phase: single launches, each with its force fields
    while (left > 0 && rr::trip_phase(s, s->istep)) {
        rr_status st = launch_steps(s, 1);
        if (st != RR_OK) return st;
        s->istep++;
        s->stepped = true;
        left--;
    }
    const int rest = left;
    if (left >= 2 * GRAPH_STEPS) {
        if (s->cur != 0) {
            rr_status st = launch_steps(s, 1);
            if (st != RR_OK) return st;
            left--;
        }
        rr_status st = build_graph(s);
        if (st != RR_OK) return st;
        while (left >= GRAPH_STEPS) {
            RR_CK(cudaGraphLaunch(s->graph, s->stream));
            left -= GRAPH_STEPS;
        }
    }
    rr_status st = launch_steps(s, left);
    if (st != RR_OK) return st;
    s->istep += rest;
    if (rest > 0) s->stepped = true;
    return RR_OK;
}

rr_status rr_sync(rr_solver *s) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    int flag = 0;
    RR_CK(cudaMemcpyAsync(&flag, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    RR_CK(cudaStreamSynchronize(s->stream));
    if (flag & rr::WATCH_STAGE_WAIT)
        return fail(RR_ERR_WATCHDOG, "watchdog %d: a wait of the staged step's pipeline timed out by step %lld",
                    flag, s->istep);
    if (flag) return fail(RR_ERR_WATCHDOG, "watchdog %d: density left (0.1, 10) or became NaN by step %lld", flag,
                          s->istep);
    return RR_OK;
}

rr_status rr_query(rr_solver *s, int *busy) {
    if (!s || !busy) return fail(RR_ERR_INVALID, "NULL argument");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    const cudaError_t e = cudaStreamQuery(s->stream);
    if (e == cudaSuccess) {
        *busy = 0;
        return RR_OK;
    }
    if (e == cudaErrorNotReady) {
        cudaGetLastError(); // not an error: work in flight
        *busy = 1;
        return RR_OK;
    }
    return fail(RR_ERR_CUDA, "cudaStreamQuery: %s", cudaGetErrorString(e));
}

rr_status rr_set_wait_limit(rr_solver *s, long long polls) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (polls > 0xFFFFFFFFll) return fail(RR_ERR_INVALID, "polls = %lld exceeds 2^32-1", polls);
    const uint32_t v = polls < 0 ? rr::STAGE_WAIT_LIMIT : (uint32_t)polls;
    if (v != s->stage_wait) {
        s->stage_wait = v;
        rr::drop_graph(s); // the captured steps carry the old limit
    }
    return RR_OK;
}

long long rr_get_wait_limit(const rr_solver *s) { return s ? (long long)s->stage_wait : -1; }

long long rr_get_istep(const rr_solver *s) { return s ? s->istep : -1; }

void *rr_get_stream(const rr_solver *s) { return s ? (void *)s->stream : nullptr; }

size_t rr_device_bytes(const rr_solver *s) { return s ? s->bytes : 0; }

rr_status rr_macro(rr_solver *s, double *rho, double *ux, double *uy, double *uz, double *taut,
                   int where) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (!s->ready) return fail(RR_ERR_STATE, "no state");
    if (!s->stepped) return fail(RR_ERR_STATE, "rr_macro needs a step after the state was set");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    rr_status st = readout_macros(s, taut != nullptr);
    if (st != RR_OK) return st;
    const size_t n = s->g.n;
    double *dst[5] = {rho, ux, uy, uz, taut};
    for (int k = 0; k < 5; k++)
        if ((st = copy_out(s, dst[k], s->aux + k * n, n, where)) != RR_OK) return st;
    return rr_sync(s);
}

rr_status rr_get_f(rr_solver *s, double *f, int where) {
    if (!s || !f) return fail(RR_ERR_INVALID, "NULL argument");
    if (!s->ready) return fail(RR_ERR_STATE, "no state");
    if (!s->stepped) return fail(RR_ERR_STATE, "rr_get_f needs a step after the state was set");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    const size_t n = s->g.n, nf = (size_t)s->p.q * n;
    double *dst = f;
    double *tmp = nullptr;
    if (where != RR_DEVICE) {
        RR_CK(cudaMallocAsync(&tmp, nf * sizeof(double), s->stream));
        dst = tmp;
    }
    cudaError_t e = readout_state(s, dst, nullptr, nullptr, nullptr, nullptr);
    if (e == cudaSuccess && tmp) e = cudaMemcpyAsync(f, tmp, nf * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (tmp) cudaFreeAsync(tmp, s->stream);
    if (e != cudaSuccess) return fail(RR_ERR_CUDA, "readout failed: %s", cudaGetErrorString(e));
    return rr_sync(s);
}

rr_status rr_diag(rr_solver *s, double out[4]) {
    if (!s || !out) return fail(RR_ERR_INVALID, "NULL argument");
    if (!s->ready || !s->stepped) return fail(RR_ERR_STATE, "rr_diag needs a step after the state was set");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    rr_status st = readout_macros(s, false);
    if (st != RR_OK) return st;
    const size_t n = s->g.n;
    double *partial = s->stat, *res = s->stat + 4 * rr::DIAG_MAX_BLOCKS;
    RR_CK(rr::launch_diag(s->g.n, s->aux + n, s->aux + 2 * n, s->aux + 3 * n, s->aux, partial, res, s->stream));
    RR_CK(cudaMemcpyAsync(out, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    return rr_sync(s);
}

static rr_status profile_device(rr_solver *s, double **prof) {
    rr_status st = readout_macros(s, s->p.use_les != 0);
    if (st != RR_OK) return st;
    const size_t n = s->g.n;
    *prof = s->stat + 4 * rr::DIAG_MAX_BLOCKS + 4;
    RR_CK(rr::launch_profile(s->g, s->p.ystar, s->aux + n, s->aux + 2 * n, s->aux + 3 * n,
                             s->p.use_les ? s->aux + 4 * n : nullptr, *prof, s->stream));
    return RR_OK;
}

rr_status rr_profile(rr_solver *s, double *out) {
    if (!s || !out) return fail(RR_ERR_INVALID, "NULL argument");
    if (!s->ready || !s->stepped) return fail(RR_ERR_STATE, "rr_profile needs a step after the state was set");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    double *prof;
    rr_status st = profile_device(s, &prof);
    if (st != RR_OK) return st;
    RR_CK(cudaMemcpyAsync(out, prof, 12 * (size_t)s->p.ly * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    return rr_sync(s);
}

rr_status rr_accumulate(rr_solver *s) {
    if (!s) return fail(RR_ERR_INVALID, "solver is NULL");
    if (!s->ready || !s->stepped) return fail(RR_ERR_STATE, "rr_accumulate needs a step after the state was set");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    double *prof;
    rr_status st = profile_device(s, &prof);
    if (st != RR_OK) return st;
    const int m = 12 * s->p.ly;
    RR_CK(rr::launch_accumulate(m, prof, prof + m, s->stream));
    s->acc_samples++;
    return RR_OK;
}

rr_status rr_get_accum(rr_solver *s, double *sums, long long *samples) {
    if (!s || !sums) return fail(RR_ERR_INVALID, "NULL argument");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    const int m = 12 * s->p.ly;
    double *acc = s->stat + 4 * rr::DIAG_MAX_BLOCKS + 4 + m;
    RR_CK(cudaMemcpyAsync(sums, acc, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (samples) *samples = s->acc_samples;
    return rr_sync(s);
}

rr_status rr_output(rr_solver *s, unsigned what, const char *dir) {
    if (!s || !dir) return fail(RR_ERR_INVALID, "NULL argument");
    rr_status st = ensure_dir(dir);
    if (st != RR_OK) return st;
    const size_t n = s->g.n;
    const std::string d(dir);
    char name[64];
    if (what & RR_OUT_DIAG) {
        // diag_flow, output.cu:37-56
        double m[4];
        if ((st = rr_diag(s, m)) != RR_OK) return st;
        printf("Step %-7lld umean = %.17e, vmean = %.17e, wmean = %.17e, rhomean = %14.6e\n", s->istep,
               m[0] / s->p.ustar, m[1], m[2], m[3]);
        fflush(stdout);
        char line[256];
        int len = snprintf(line, sizeof line, "%-7lld %14.6e %14.6e %14.6e %14.6e\n", s->istep, m[0], m[1], m[2], m[3]);
        if ((st = write_file(d + "/statistics.dat", line, (size_t)len, "a")) != RR_OK) return st;
    }
    if (what & (RR_OUT_FLOW)) {
        // output_flow, output.cu:89-131: rho, ux, uy, uz FP64 back to back
        std::vector<double> h(4 * n);
        if ((st = rr_macro(s, h.data(), h.data() + n, h.data() + 2 * n, h.data() + 3 * n, nullptr, RR_HOST)) != RR_OK)
            return st;
        snprintf(name, sizeof name, "/%09lld.dat", s->istep);
        if ((st = write_file(d + name, h.data(), 4 * n * sizeof(double), "wb")) != RR_OK) return st;
    }
    if (what & RR_OUT_PROFILE) {
        // output_profile, output.cu:158-214.  The reference passes iy + 0.5 to
        // a "%d" conversion (output.cu:213-214): on x86-64 and aarch64 the %d
        // then reads an unrelated integer register and the eleven %e
        // conversions print the first eleven doubles (iy + 0.5 ... <v'w'>),
        // leaving <tau_t> unprinted.  Those are the columns written here, with
        // iy in place of the unspecified integer; rr_profile() returns <tau_t>.
        std::vector<double> pr(12 * (size_t)s->p.ly);
        if ((st = rr_profile(s, pr.data())) != RR_OK) return st;
        std::string txt = std::to_string(s->istep) + "\n";
        char line[512];
        for (int iy = 0; iy < s->p.ly; iy++) {
            const double *o = pr.data() + 11 * (size_t)iy;
            snprintf(line, sizeof line,
                     "%d, %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e\n", iy,
                     o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], o[9], o[10]);
            txt += line;
        }
        if ((st = write_file(d + "/Profiles.txt", txt.data(), txt.size(), "a")) != RR_OK) return st;
    }
    if (what & RR_OUT_F) {
        // output_f, output.cu:227-258
        std::vector<double> h((size_t)s->p.q * n);
        if ((st = rr_get_f(s, h.data(), RR_HOST)) != RR_OK) return st;
        snprintf(name, sizeof name, "/f%09lld.dat", s->istep);
        if ((st = write_file(d + name, h.data(), h.size() * sizeof(double), "wb")) != RR_OK) return st;
    }
    return RR_OK;
}

rr_status rr_get_force(rr_solver *s, double *out, int where) {
    if (!s || !out) return fail(RR_ERR_INVALID, "NULL argument");
    if (!s->ready) return fail(RR_ERR_STATE, "rr_get_force before rr_init_state / rr_load");
    if (set_device(s) != RR_OK) return RR_ERR_CUDA;
    const size_t n = s->g.n;
    const double *ff = readout_field(s);
    if (!ff && s->ffield && s->istep == 0 && s->p.trip_steps > 1) ff = rr::trip_slot(s, 1); // before step 1
    if (ff) {
        const cudaMemcpyKind kind = where == RR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        for (int c = 0; c < 3; c++)
            RR_CK(cudaMemcpyAsync(out + c * n, ff + (size_t)c * s->g.stride, n * sizeof(double), kind, s->stream));
        if (where != RR_DEVICE) RR_CK(cudaStreamSynchronize(s->stream));
        return RR_OK;
    }
    if (where == RR_DEVICE) {
        std::vector<double> h(3 * n);
        for (int c = 0; c < 3; c++) std::fill(h.begin() + c * n, h.begin() + (c + 1) * n, s->p.force[c]);
        RR_CK(cudaMemcpyAsync(out, h.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        RR_CK(cudaStreamSynchronize(s->stream));
    } else {
        RR_CK(cudaStreamSynchronize(s->stream));
        for (int c = 0; c < 3; c++) std::fill(out + c * n, out + (c + 1) * n, s->p.force[c]);
    }
    return RR_OK;
}

rr_status rr_save(rr_solver *s, const char *dir) { return rr_output(s, RR_OUT_FLOW | RR_OUT_F, dir); }

rr_status rr_load(rr_solver *s, const char *dir, long long istep) {
    // initialize() with CONTINUE_STEP > 0, initial.cu:189-265
    if (!s || !dir) return fail(RR_ERR_INVALID, "NULL argument");
    if (s->batch) return fail(RR_ERR_STATE, "the solver is a member of a batch: remove it to set its state");
    const size_t n = s->g.n, nf = (size_t)s->p.q * n;
    std::vector<double> m(4 * n), f(nf);
    char name[64];
    auto rd = [&](const std::string &path, double *dst, size_t count) -> rr_status {
        FILE *fp = fopen(path.c_str(), "rb");
        if (!fp) return fail(RR_ERR_IO, "cannot open file: %s", path.c_str());
        size_t r = fread(dst, sizeof(double), count, fp);
        fclose(fp);
        if (r != count) return fail(RR_ERR_IO, "%s: read %zu of %zu elements", path.c_str(), r, count);
        return RR_OK;
    };
    snprintf(name, sizeof name, "/%09lld.dat", istep);
    rr_status st = rd(std::string(dir) + name, m.data(), 4 * n);
    if (st != RR_OK) return st;
    snprintf(name, sizeof name, "/f%09lld.dat", istep);
    if ((st = rd(std::string(dir) + name, f.data(), nf)) != RR_OK) return st;
    return init_state_at(s, f.data(), m.data(), m.data() + n, m.data() + 2 * n, m.data() + 3 * n, RR_HOST, istep);
}

} // extern "C"
