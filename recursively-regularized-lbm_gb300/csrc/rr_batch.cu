// rr_batch.cu -- batches of domains and the launch-shape autotuner.
//
// A batch keeps every member's state where it already lives (the member
// solver's two population buffers) and advances all members together:
// members whose step is the tile step are grouped by (storage, lattice,
// forcing) class, and each class takes one persistent batch_kernel launch per
// step over a device table of the members' tile descriptors; the other
// members (WALE, lx < 3) add their own launch.  The descriptor of a member
// points at its buffers for one buffer parity, so the batch keeps every
// member on the same parity (a member joining on the other parity has its two
// buffer labels swapped, which moves no data) and holds two tables.
//
// The autotuner times launch shapes on real steps.  No shape changes any
// result: the per-node arithmetic and rounding stream of a node do not depend
// on which warp or CTA computes it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "rr_internal.h"

namespace {

constexpr int BATCH_GRAPH_STEPS = 32; // steps per captured graph (even: ends on the same parity)
constexpr int MAX_CHAINS = 32;        // fan-out mode: most parallel chains

#define BK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return rr_internal_error(RR_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                 \
                                     cudaGetErrorString(e_), __FILE__, __LINE__);                 \
    } while (0)

// members that share one persistent launch: one (storage, lattice, forcing)
// class, and either members small enough to stay in L2 together or the rest
struct Class {
    const rr::Ops *ops = nullptr;
    int q = 27;
    bool force = false;
    std::vector<rr_solver *> members;
    void *desc[2] = {nullptr, nullptr}; // device descriptor tables, per parity
    uint32_t *cta_begin = nullptr;      // device [members + 1]
    uint32_t *cta_dom = nullptr;        // device [total_ctas]: member of each CTA
    uint32_t total_ctas = 0;
    int grid = 0;
    size_t bytes = 0; // population buffers of the members
};

__global__ void gather_status(int *const *ptrs, int n, int *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = *ptrs[i];
}

} // namespace

struct rr_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<rr_solver *> members; // in order of addition
    int parity = 0;                   // cur of every member
    bool dirty = true;                // tables and graph must be rebuilt
    std::vector<Class> classes;
    std::vector<rr_solver *> others; // members stepped by their own launch
    cudaGraphExec_t graph = nullptr;
    int block = 256, ctas_per_sm = 0;
    int order = 0; // 0: strided walk over the CTAs, 1: contiguous chunks
    size_t group_bytes = 0; // members whose buffers fit are grouped up to this size and run
                            // their steps back to back (L2 reuse); 0: no grouping
    int mode = RR_BATCH_PERSISTENT;
    int chains = 8;                                 // fan-out mode: parallel chains
    std::vector<cudaStream_t> side;                 // one stream per chain
    std::vector<cudaEvent_t> side_done;             // one event per chain
    cudaEvent_t fork = nullptr;
    std::vector<std::vector<rr_solver *>> chain;    // members of each chain
    int sms = 0;
    int **status_ptrs = nullptr; // device: every member's watchdog word
    int *status_vals = nullptr;  // device
    int *status_host = nullptr;  // pinned
    int status_cap = 0;
};

namespace {

void drop_tables(rr_batch *b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    for (Class &c : b->classes) {
        cudaFree(c.desc[0]);
        cudaFree(c.desc[1]);
        cudaFree(c.cta_begin);
        cudaFree(c.cta_dom);
    }
    b->classes.clear();
    b->others.clear();
}

rr_status build_tables(rr_batch *b) {
    if (!b->dirty) return RR_OK;
    BK(cudaStreamSynchronize(b->stream)); // the old tables may still be read
    drop_tables(b);
    // per class: members larger than group_bytes share one launch group; the
    // others are packed, in order of addition, into groups of at most
    // group_bytes of population buffers
    std::vector<Class> big;
    for (rr_solver *s : b->members) {
        if (!rr::batchable(s)) {
            b->others.push_back(s);
            continue;
        }
        const bool force = rr::has_force(s->p);
        const size_t fb = 2 * (size_t)s->p.q * s->g.stride * s->ops->elem_bytes;
        const bool small = b->group_bytes > 0 && fb <= b->group_bytes;
        std::vector<Class> &pool = small ? b->classes : big;
        auto it = std::find_if(pool.begin(), pool.end(), [&](const Class &c) {
            return c.ops == s->ops && c.q == s->p.q && c.force == force && (!small || c.bytes + fb <= b->group_bytes);
        });
        if (it == pool.end()) {
            Class c;
            c.ops = s->ops;
            c.q = s->p.q;
            c.force = force;
            pool.push_back(c);
            it = pool.end() - 1;
        }
        it->members.push_back(s);
        it->bytes += fb;
    }
    b->classes.insert(b->classes.end(), big.begin(), big.end());
    for (Class &c : b->classes) {
        const size_t nd = c.members.size();
        const rr_solver *s0 = c.members[0];
        const size_t dsz = c.ops->tile_desc(c.q, nullptr, nullptr, s0->g, 0.0, s0->p.force, nullptr, nullptr, 0,
                                            32, nullptr, nullptr);
        std::vector<unsigned char> h[2] = {std::vector<unsigned char>(nd * dsz),
                                           std::vector<unsigned char>(nd * dsz)};
        std::vector<uint32_t> begin(nd + 1, 0);
        for (size_t k = 0; k < nd; k++) {
            rr_solver *s = c.members[k];
            uint32_t nitems = 0;
            for (int p = 0; p < 2; p++)
                c.ops->tile_desc(c.q, s->buf[p], s->buf[1 - p], s->g, 1.0 - 1.0 / s->p.tau, s->p.force, s->status,
                                 s->edge_list, s->nedges, s->rows_group, h[p].data() + k * dsz, &nitems);
            const unsigned long long ctas = ((unsigned long long)nitems * 32ull + b->block - 1) / b->block;
            if ((unsigned long long)begin[k] + ctas > 0xFFFFFFFFull)
                return rr_internal_error(RR_ERR_INVALID, "batch has more than 2^32 CTAs of work");
            begin[k + 1] = begin[k] + (uint32_t)ctas;
        }
        c.total_ctas = begin[nd];
        for (int p = 0; p < 2; p++) {
            if (cudaMalloc(&c.desc[p], nd * dsz) != cudaSuccess) {
                cudaGetLastError();
                c.desc[p] = nullptr;
                return rr_internal_error(RR_ERR_NOMEM, "cannot allocate the batch descriptors");
            }
            BK(cudaMemcpy(c.desc[p], h[p].data(), nd * dsz, cudaMemcpyHostToDevice));
        }
        if (cudaMalloc(&c.cta_begin, (nd + 1) * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            c.cta_begin = nullptr;
            return rr_internal_error(RR_ERR_NOMEM, "cannot allocate the batch CTA table");
        }
        BK(cudaMemcpy(c.cta_begin, begin.data(), (nd + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice));
        std::vector<uint32_t> dom(c.total_ctas);
        for (size_t k = 0; k < nd; k++)
            std::fill(dom.begin() + begin[k], dom.begin() + begin[k + 1], (uint32_t)k);
        if (cudaMalloc(&c.cta_dom, std::max<size_t>(dom.size(), 1) * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            c.cta_dom = nullptr;
            return rr_internal_error(RR_ERR_NOMEM, "cannot allocate the batch CTA map");
        }
        if (!dom.empty()) BK(cudaMemcpy(c.cta_dom, dom.data(), dom.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        const int occ = c.ops->batch_occupancy(c.q, c.force, b->block);
        if (occ <= 0) return rr_internal_error(RR_ERR_CUDA, "batch kernel occupancy query failed");
        const int cps = b->ctas_per_sm > 0 ? std::min(b->ctas_per_sm, occ) : occ;
        c.grid = (int)std::min<unsigned long long>(c.total_ctas, (unsigned long long)cps * b->sms);
        if (c.grid < 1) c.grid = 1;
    }
    // fan-out chains: members by decreasing size, each to the least loaded chain
    b->chain.assign(b->chains, {});
    {
        std::vector<rr_solver *> order(b->members);
        std::stable_sort(order.begin(), order.end(), [](const rr_solver *x, const rr_solver *y) {
            return (size_t)x->g.n * x->ops->elem_bytes > (size_t)y->g.n * y->ops->elem_bytes;
        });
        std::vector<double> load(b->chains, 0.0);
        for (rr_solver *s : order) {
            const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            b->chain[c].push_back(s);
            load[c] += (double)s->g.n * (s->p.use_les ? 2.0 : 1.0) * (double)s->ops->elem_bytes;
        }
    }
    // watchdog gather table
    const int n = (int)b->members.size();
    if (n > b->status_cap) {
        cudaFree(b->status_ptrs);
        cudaFree(b->status_vals);
        cudaFreeHost(b->status_host);
        b->status_ptrs = nullptr;
        b->status_vals = nullptr;
        b->status_host = nullptr;
        b->status_cap = 0;
        const int cap = std::max(n, 2 * b->status_cap);
        if (cudaMalloc(&b->status_ptrs, cap * sizeof(int *)) != cudaSuccess ||
            cudaMalloc(&b->status_vals, cap * sizeof(int)) != cudaSuccess ||
            cudaMallocHost(&b->status_host, cap * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return rr_internal_error(RR_ERR_NOMEM, "cannot allocate the batch watchdog table");
        }
        b->status_cap = cap;
    }
    if (n > 0) {
        std::vector<int *> ptrs(n);
        for (int k = 0; k < n; k++) ptrs[k] = b->members[k]->status;
        BK(cudaMemcpy(b->status_ptrs, ptrs.data(), n * sizeof(int *), cudaMemcpyHostToDevice));
    }
    b->dirty = false;
    return RR_OK;
}

// n steps of every member from buffer parity p, group after group (a group's
// steps run back to back, so a group that fits in L2 stays there)
rr_status launch_batch_steps(rr_batch *b, int p, int n) {
    if (b->mode == RR_BATCH_FANOUT) {
        // every chain forks from the batch stream, runs its members' n steps
        // member after member, and joins back
        BK(cudaEventRecord(b->fork, b->stream));
        for (int c = 0; c < b->chains; c++) {
            if (b->chain[c].empty()) continue;
            BK(cudaStreamWaitEvent(b->side[c], b->fork, 0));
            for (rr_solver *s : b->chain[c])
                for (int k = 0; k < n; k++) {
                    const int q = p ^ (k & 1);
                    rr_status st = rr::launch_one(s, s->buf[q], s->buf[1 - q], b->side[c]);
                    if (st != RR_OK) return st;
                }
            BK(cudaEventRecord(b->side_done[c], b->side[c]));
            BK(cudaStreamWaitEvent(b->stream, b->side_done[c], 0));
        }
        return RR_OK;
    }
    for (Class &c : b->classes)
        for (int k = 0; k < n; k++) {
            const int q = p ^ (k & 1);
            BK(c.ops->batch(c.q, c.force, c.desc[q], c.cta_begin, c.cta_dom, (uint32_t)c.members.size(),
                            c.total_ctas, b->block, c.grid, b->order, b->stream));
        }
    for (rr_solver *s : b->others)
        for (int k = 0; k < n; k++) {
            const int q = p ^ (k & 1);
            rr_status st = rr::launch_one(s, s->buf[q], s->buf[1 - q], b->stream);
            if (st != RR_OK) return st;
        }
    return RR_OK;
}

rr_status build_graph(rr_batch *b) {
    if (b->graph) return RR_OK;
    cudaGraph_t graph;
    BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    rr_status st = RR_OK;
    st = launch_batch_steps(b, 0, BATCH_GRAPH_STEPS);
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (st != RR_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return rr_internal_error(RR_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return rr_internal_error(RR_ERR_CUDA, "batch graph instantiate failed: %s", cudaGetErrorString(e));
    }
    return RR_OK;
}

// ---- autotuner records, per size class ----
using TuneKey = std::tuple<int, int, int, int, int>; // q, storage, les, force, log2 class
std::mutex g_tune_mu;
std::map<TuneKey, int> g_rows_group;
std::map<TuneKey, rr::LesTile> g_les_tile;
struct StageShape {
    int method, rows, stages;
};
std::map<TuneKey, StageShape> g_stage;

TuneKey tune_key(const rr_params &p) {
    const double n = (double)p.lx * p.ly * p.lz;
    const int cls = (int)std::ceil(std::log2(std::max(n, 1.0)));
    return TuneKey{p.q, p.storage, p.use_les ? 1 : 0, rr::has_force(p) ? 1 : 0, cls};
}

// milliseconds of `steps` steps of fn on stream st (CUDA events)
template <class Fn>
rr_status time_steps(cudaStream_t st, Fn fn, float *ms) {
    cudaEvent_t e0, e1;
    BK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return rr_internal_error(RR_ERR_CUDA, "cudaEventCreate failed");
    }
    rr_status r = RR_OK;
    cudaError_t e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) r = fn();
    if (e == cudaSuccess && r == RR_OK) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess && r == RR_OK) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess && r == RR_OK) e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r != RR_OK) return r;
    if (e != cudaSuccess) return rr_internal_error(RR_ERR_CUDA, "timing failed: %s", cudaGetErrorString(e));
    return RR_OK;
}

} // namespace

namespace rr {

bool tuned_rows_group(const rr_params &p, int *rows_group) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_rows_group.find(tune_key(p));
    if (it == g_rows_group.end()) return false;
    *rows_group = it->second;
    return true;
}

bool tuned_stage(const rr_params &p, int *method, int *rows, int *stages) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_stage.find(tune_key(p));
    if (it == g_stage.end()) return false;
    *method = it->second.method;
    *rows = it->second.rows;
    *stages = it->second.stages;
    return true;
}

bool tuned_les_tile(const rr_params &p, LesTile *tile) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_les_tile.find(tune_key(p));
    if (it == g_les_tile.end()) return false;
    *tile = it->second;
    return true;
}

rr_status batch_detach(rr_solver *s) { return rr_batch_remove(s->batch, s); }

} // namespace rr

extern "C" {

rr_status rr_batch_create(int device, rr_batch **out) {
    if (!out) return rr_internal_error(RR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    BK(cudaSetDevice(device));
    rr_batch *b = new rr_batch;
    b->device = device;
    int l2 = 0;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device) != cudaSuccess) {
        cudaGetLastError();
        if (b->stream) cudaStreamDestroy(b->stream);
        delete b;
        return rr_internal_error(RR_ERR_CUDA, "batch stream creation failed");
    }
    b->group_bytes = 0;
    b->side.assign(MAX_CHAINS, nullptr);
    b->side_done.assign(MAX_CHAINS, nullptr);
    bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int c = 0; c < MAX_CHAINS && ok; c++)
        ok = cudaStreamCreateWithFlags(&b->side[c], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->side_done[c], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        rr_batch_destroy(b);
        return rr_internal_error(RR_ERR_CUDA, "batch stream creation failed");
    }
    *out = b;
    return RR_OK;
}

rr_status rr_batch_destroy(rr_batch *b) {
    if (!b) return RR_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    while (!b->members.empty()) rr_batch_remove(b, b->members.back());
    drop_tables(b);
    cudaFree(b->status_ptrs);
    cudaFree(b->status_vals);
    cudaFreeHost(b->status_host);
    for (cudaStream_t st : b->side)
        if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->side_done)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    cudaStreamDestroy(b->stream);
    cudaGetLastError();
    delete b;
    return RR_OK;
}

rr_status rr_batch_add(rr_batch *b, rr_solver *s) {
    if (!b || !s) return rr_internal_error(RR_ERR_INVALID, "NULL argument");
    if (s->batch) return rr_internal_error(RR_ERR_STATE, "the solver is already a member of a batch");
    if (!s->ready) return rr_internal_error(RR_ERR_STATE, "the solver has no state (rr_init_state / rr_load)");
    if (rr::trip_phase(s, s->istep))
        return rr_internal_error(RR_ERR_STATE, "the solver is in its trip-forcing phase (until step %d)",
                                 s->p.trip_steps);
    if (s->p.device != b->device)
        return rr_internal_error(RR_ERR_INVALID, "solver on device %d, batch on device %d", s->p.device, b->device);
    BK(cudaSetDevice(b->device));
    BK(cudaStreamSynchronize(s->stream)); // the solver's own pending work
    if (s->cur != b->parity) {
        std::swap(s->buf[0], s->buf[1]);
        std::swap(s->fdbc_wt[0], s->fdbc_wt[1]);
        s->cur = b->parity;
        rr::drop_graph(s); // captured with the old labels
    }
    s->stream = b->stream;
    s->batch = b;
    b->members.push_back(s);
    b->dirty = true;
    return RR_OK;
}

rr_status rr_batch_remove(rr_batch *b, rr_solver *s) {
    if (!b || !s) return rr_internal_error(RR_ERR_INVALID, "NULL argument");
    auto it = std::find(b->members.begin(), b->members.end(), s);
    if (it == b->members.end() || s->batch != b) return rr_internal_error(RR_ERR_INVALID, "not a member of this batch");
    cudaSetDevice(b->device);
    BK(cudaStreamSynchronize(b->stream));
    s->stream = s->home;
    s->batch = nullptr;
    b->members.erase(it);
    b->dirty = true;
    return RR_OK;
}

int rr_batch_size(const rr_batch *b) { return b ? (int)b->members.size() : 0; }

void *rr_batch_get_stream(const rr_batch *b) { return b ? (void *)b->stream : nullptr; }

rr_status rr_batch_step(rr_batch *b, int nsteps) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (nsteps < 0) return rr_internal_error(RR_ERR_INVALID, "nsteps = %d", nsteps);
    if (b->members.empty() || nsteps == 0) return RR_OK;
    BK(cudaSetDevice(b->device));
    rr_status st = build_tables(b);
    if (st != RR_OK) return st;
    int left = nsteps;
    if (left >= 2 * BATCH_GRAPH_STEPS) {
        if (b->parity != 0) {
            if ((st = launch_batch_steps(b, 1, 1)) != RR_OK) return st;
            b->parity = 0;
            left--;
        }
        if ((st = build_graph(b)) != RR_OK) return st;
        while (left >= BATCH_GRAPH_STEPS) {
            BK(cudaGraphLaunch(b->graph, b->stream));
            left -= BATCH_GRAPH_STEPS;
        }
    }
    if (left > 0) {
        if ((st = launch_batch_steps(b, b->parity, left)) != RR_OK) return st;
        b->parity ^= left & 1;
    }
    for (rr_solver *s : b->members) {
        s->cur = b->parity;
        s->istep += nsteps;
        s->stepped = true;
    }
    return RR_OK;
}

rr_status rr_batch_sync(rr_batch *b) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    BK(cudaSetDevice(b->device));
    const int n = (int)b->members.size();
    if (n == 0) {
        BK(cudaStreamSynchronize(b->stream));
        return RR_OK;
    }
    rr_status st = build_tables(b);
    if (st != RR_OK) return st;
    gather_status<<<(n + 255) / 256, 256, 0, b->stream>>>(b->status_ptrs, n, b->status_vals);
    BK(cudaGetLastError());
    BK(cudaMemcpyAsync(b->status_host, b->status_vals, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int k = 0; k < n; k++)
        if (b->status_host[k])
            return rr_internal_error(RR_ERR_WATCHDOG,
                                     (b->status_host[k] & rr::WATCH_STAGE_WAIT)
                                         ? "watchdog %d: a pipeline wait timed out in batch member %d (step <= %lld)"
                                         : "watchdog %d: density out of range or NaN in batch member %d (step <= %lld)",
                                     b->status_host[k], k, b->members[k]->istep);
    return RR_OK;
}

rr_status rr_batch_set_launch(rr_batch *b, int block, int ctas_per_sm, int order) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (block != 64 && block != 128 && block != 256)
        return rr_internal_error(RR_ERR_INVALID, "block = %d, must be 64, 128 or 256", block);
    if (ctas_per_sm < 0) return rr_internal_error(RR_ERR_INVALID, "ctas_per_sm = %d", ctas_per_sm);
    if (order != RR_BATCH_STRIDED && order != RR_BATCH_CHUNKED)
        return rr_internal_error(RR_ERR_INVALID, "order = %d unknown", order);
    if (block != b->block || ctas_per_sm != b->ctas_per_sm || order != b->order) {
        b->block = block;
        b->ctas_per_sm = ctas_per_sm;
        b->order = order;
        b->dirty = true;
    }
    return RR_OK;
}

rr_status rr_batch_get_launch(const rr_batch *b, int *block, int *ctas_per_sm, int *order) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (block) *block = b->block;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    if (order) *order = b->order;
    return RR_OK;
}

rr_status rr_batch_set_mode(rr_batch *b, int mode, int chains) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (mode != RR_BATCH_PERSISTENT && mode != RR_BATCH_FANOUT)
        return rr_internal_error(RR_ERR_INVALID, "mode = %d unknown", mode);
    if (chains < 1 || chains > MAX_CHAINS)
        return rr_internal_error(RR_ERR_INVALID, "chains = %d, must be 1 to %d", chains, MAX_CHAINS);
    if (mode != b->mode || chains != b->chains) {
        b->mode = mode;
        b->chains = chains;
        b->dirty = true;
    }
    return RR_OK;
}

rr_status rr_batch_get_mode(const rr_batch *b, int *mode, int *chains) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (mode) *mode = b->mode;
    if (chains) *chains = b->chains;
    return RR_OK;
}

rr_status rr_batch_set_grouping(rr_batch *b, size_t group_bytes) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (group_bytes != b->group_bytes) {
        b->group_bytes = group_bytes;
        b->dirty = true;
    }
    return RR_OK;
}

size_t rr_batch_get_grouping(const rr_batch *b) { return b ? b->group_bytes : 0; }

rr_status rr_get_launch(const rr_solver *s, int *rows_group, int *les_method, int les_tile[3]) {
    if (!s) return rr_internal_error(RR_ERR_INVALID, "solver is NULL");
    if (rows_group) *rows_group = s->rows_group;
    if (les_method) *les_method = s->les_method;
    if (les_tile) {
        les_tile[0] = s->tile.tx;
        les_tile[1] = s->tile.ty;
        les_tile[2] = s->tile.zchunk;
    }
    return RR_OK;
}

rr_status rr_set_launch(rr_solver *s, int rows_group, const int *les_method, const int les_tile[3]) {
    if (!s) return rr_internal_error(RR_ERR_INVALID, "solver is NULL");
    int method = s->les_method;
    if (les_method) {
        method = *les_method;
        if (method != RR_LES_FUSED && method != RR_LES_TWO_PASS)
            return rr_internal_error(RR_ERR_INVALID, "les_method = %d unknown", method);
        if (method == RR_LES_TWO_PASS && !s->ubuf)
            return rr_internal_error(RR_ERR_INVALID, "the two-pass WALE step needs use_les and lx >= 3");
        if (method == RR_LES_FUSED && s->fdbc && s->p.use_les)
            return rr_internal_error(RR_ERR_UNSUPPORTED, "WALE with the finite-difference closure is two-pass only");
    }
    if (rows_group < 32 || rows_group % 32 != 0 || rows_group > 4096)
        return rr_internal_error(RR_ERR_INVALID, "rows_group = %d, must be a multiple of 32 in [32, 4096]", rows_group);
    rr::LesTile t = s->tile;
    if (les_tile) {
        t.tx = les_tile[0];
        t.ty = les_tile[1];
        t.zchunk = les_tile[2];
        if (t.tx < 1 || t.ty < 1 || t.tx * t.ty > 256 || t.tx % 32 != 0 && t.tx * t.ty % 32 != 0 || t.zchunk < 1)
            return rr_internal_error(RR_ERR_INVALID, "WALE tile %dx%d (z chunk %d): need tx*ty <= 256, a multiple of 32",
                                     t.tx, t.ty, t.zchunk);
    }
    if (rows_group != s->rows_group || t.tx != s->tile.tx || t.ty != s->tile.ty || t.zchunk != s->tile.zchunk ||
        method != s->les_method) {
        s->rows_group = rows_group;
        s->tile = t;
        s->les_method = method;
        rr::drop_graph(s);
        if (s->batch) s->batch->dirty = true;
    }
    return RR_OK;
}

rr_status rr_set_stage(rr_solver *s, int method, int rows, int stages) {
    if (!s) return rr_internal_error(RR_ERR_INVALID, "solver is NULL");
    if (method != RR_DNS_TILE && method != RR_DNS_STAGED)
        return rr_internal_error(RR_ERR_INVALID, "method = %d unknown", method);
    if (method == RR_DNS_STAGED) {
        if (!s->frow_list)
            return rr_internal_error(RR_ERR_INVALID, "the staged step needs a DNS grid of at least 3 nodes per axis "
                                                     "with rows a multiple of 16 bytes");
        const int rmax = std::min(32, s->p.ly - 2);
        if (rows < 1 || rows > rmax || stages < 2 || stages > 4)
            return rr_internal_error(RR_ERR_INVALID, "rows = %d (1 .. %d), stages = %d (2 .. 4)", rows, rmax, stages);
        const size_t wall = s->p.face[0] != RR_FACE_PERIODIC ? (size_t)stages * 2 * s->p.q * rows * s->ops->elem_bytes : 0;
        const size_t smem = 128 + (size_t)stages * s->p.q * rows * s->p.lx * s->ops->elem_bytes + wall;
        if (smem > 227 * 1024)
            return rr_internal_error(RR_ERR_INVALID, "%d stages of %d rows need %zu bytes of shared memory (> 227 KB)",
                                     stages, rows, smem);
        s->stage_rows = rows;
        s->stages = stages;
    }
    if (method != s->dns_method) {
        s->dns_method = method;
        rr::drop_graph(s);
    }
    return RR_OK;
}

rr_status rr_get_stage(const rr_solver *s, int *method, int *rows, int *stages) {
    if (!s) return rr_internal_error(RR_ERR_INVALID, "solver is NULL");
    if (method) *method = s->dns_method;
    if (rows) *rows = s->stage_rows;
    if (stages) *stages = s->stages;
    return RR_OK;
}

rr_status rr_tune(rr_solver *s, int trial_steps, long long *steps_run) {
    if (!s) return rr_internal_error(RR_ERR_INVALID, "solver is NULL");
    if (trial_steps < 1) return rr_internal_error(RR_ERR_INVALID, "trial_steps = %d", trial_steps);
    if (s->batch) return rr_internal_error(RR_ERR_STATE, "the solver is a member of a batch: use rr_batch_tune");
    if (!s->ready) return rr_internal_error(RR_ERR_STATE, "rr_tune before rr_init_state / rr_load");
    long long run = 0;
    auto step = [&](int n) -> rr_status {
        rr_status r = rr_step(s, n);
        if (r == RR_OK) run += n;
        return r;
    };
    rr_status st = step(1); // first launches (module load) outside the timings
    if (st != RR_OK) return st;
    const int trial = std::min(trial_steps, 63); // plain launches, no graph capture per candidate
    if (s->p.use_les && s->les_method == RR_LES_FUSED) {
        // the fused WALE step: x-y tile and z chunk.  (The two WALE methods
        // round differently in FP32, so the method is the caller's choice and
        // the tuner keeps it.)
        std::vector<rr::LesTile> cands;
        const int zcs[3] = {8, 16, 32};
        const int shapes[4][2] = {{32, 8}, {64, 4}, {32, 4}, {16, 16}};
        for (auto &sh : shapes)
            for (int zc : zcs)
                if (zc <= std::max(8, s->p.lz)) cands.push_back(rr::LesTile{sh[0], sh[1], zc});
        float best = 1e30f;
        rr::LesTile bt = s->tile;
        for (const rr::LesTile &t : cands) {
            s->tile = t;
            float ms = 0;
            if ((st = time_steps(s->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
            if (ms < best) {
                best = ms;
                bt = t;
            }
        }
        s->tile = bt;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_les_tile[tune_key(s->p)] = bt;
    } else if (rr::tile_step(s) || s->les_method == RR_LES_TWO_PASS) {
        // the tile step, or the two tile passes of the WALE step: rows per
        // group; then (DNS) the staged step's block rows and stages
        const int method0 = s->dns_method;
        s->dns_method = RR_DNS_TILE;
        const int cands[3] = {32, 64, 128};
        float best = 1e30f;
        int br = s->rows_group;
        for (int rg : cands) {
            s->rows_group = rg;
            float ms = 0;
            if ((st = time_steps(s->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
            if (ms < best) {
                best = ms;
                br = rg;
            }
        }
        s->rows_group = br;
        StageShape bs{RR_DNS_TILE, s->stage_rows, s->stages};
        if (s->frow_list) {
            const int r0 = s->stage_rows;
            const StageShape cs[4] = {{RR_DNS_STAGED, r0, 2}, {RR_DNS_STAGED, std::max(1, r0 / 2), 2},
                                      {RR_DNS_STAGED, std::max(1, r0 / 2), 3}, {RR_DNS_STAGED, 2 * r0, 2}};
            for (const StageShape &c : cs) {
                if (rr_set_stage(s, c.method, c.rows, c.stages) != RR_OK) continue;
                float ms = 0;
                if ((st = time_steps(s->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
                if (ms < best) {
                    best = ms;
                    bs = c;
                }
            }
        }
        (void)method0;
        if (bs.method == RR_DNS_STAGED) {
            rr_set_stage(s, bs.method, bs.rows, bs.stages);
        } else {
            s->dns_method = RR_DNS_TILE;
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_rows_group[tune_key(s->p)] = br;
        if (s->frow_list) g_stage[tune_key(s->p)] = StageShape{s->dns_method, s->stage_rows, s->stages};
    }
    rr::drop_graph(s);
    if (steps_run) *steps_run = run;
    return RR_OK;
}

rr_status rr_batch_tune(rr_batch *b, int trial_steps, long long *steps_run) {
    if (!b) return rr_internal_error(RR_ERR_INVALID, "batch is NULL");
    if (trial_steps < 1) return rr_internal_error(RR_ERR_INVALID, "trial_steps = %d", trial_steps);
    long long run = 0;
    if (b->members.empty()) {
        if (steps_run) *steps_run = 0;
        return RR_OK;
    }
    const int trial = std::min(trial_steps, 2 * BATCH_GRAPH_STEPS - 1); // plain launches
    auto step = [&](int n) -> rr_status {
        rr_status r = rr_batch_step(b, n);
        if (r == RR_OK) run += n;
        return r;
    };
    rr_status st = step(1);
    if (st != RR_OK) return st;
    // 0. fan-out chains (the members' own launches on parallel graph branches)
    float best_fan = 1e30f;
    int best_chains = b->chains;
    for (int ch : {4, 8, 16}) {
        if ((st = rr_batch_set_mode(b, RR_BATCH_FANOUT, ch)) != RR_OK) return st;
        float ms = 0;
        if ((st = time_steps(b->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
        if (ms < best_fan) {
            best_fan = ms;
            best_chains = ch;
        }
    }
    if ((st = rr_batch_set_mode(b, RR_BATCH_PERSISTENT, best_chains)) != RR_OK) return st;
    // 1. threads per CTA and CTAs per SM of the persistent launch
    int occ_max = 0;
    for (rr_solver *s : b->members)
        if (rr::batchable(s)) occ_max = std::max(occ_max, s->ops->batch_occupancy(s->p.q, rr::has_force(s->p), 128));
    struct Shape {
        int block, cps, order;
    };
    std::vector<Shape> shapes;
    for (int order : {RR_BATCH_STRIDED, RR_BATCH_CHUNKED})
        for (int block : {128, 256}) {
            const int occ = std::max(1, block == 128 ? occ_max : occ_max / 2);
            shapes.push_back(Shape{block, 0, order});
            if (occ / 2 >= 1 && occ / 2 != occ) shapes.push_back(Shape{block, occ / 2, order});
        }
    float best = 1e30f;
    Shape bs{b->block, b->ctas_per_sm, b->order};
    for (const Shape &sh : shapes) {
        if ((st = rr_batch_set_launch(b, sh.block, sh.cps, sh.order)) != RR_OK) return st;
        float ms = 0;
        if ((st = time_steps(b->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
        if (ms < best) {
            best = ms;
            bs = sh;
        }
    }
    if ((st = rr_batch_set_launch(b, bs.block, bs.cps, bs.order)) != RR_OK) return st;
    // 2. L2 grouping of the small members: none, a quarter, half of L2
    {
        int l2 = 0;
        BK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device));
        const size_t cands[3] = {0, (size_t)l2 / 4, (size_t)l2 / 2};
        size_t bg = b->group_bytes;
        float bt = 1e30f;
        for (size_t gb : cands) {
            if ((st = rr_batch_set_grouping(b, gb)) != RR_OK) return st;
            float ms = 0;
            if ((st = time_steps(b->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
            if (ms < bt) {
                bt = ms;
                bg = gb;
            }
        }
        if ((st = rr_batch_set_grouping(b, bg)) != RR_OK) return st;
        if (best_fan < std::min(best, bt)) {
            if ((st = rr_batch_set_mode(b, RR_BATCH_FANOUT, best_chains)) != RR_OK) return st;
        }
    }
    // 3. rows per work-item group, per size class of the tile-step members
    std::map<TuneKey, std::vector<rr_solver *>> by_class;
    for (rr_solver *s : b->members)
        if (rr::tile_step(s)) by_class[tune_key(s->p)].push_back(s);
    for (auto &kv : by_class) {
        int br = kv.second[0]->rows_group;
        float bt = 1e30f;
        for (int rg : {32, 64, 128}) {
            for (rr_solver *s : kv.second) s->rows_group = rg;
            b->dirty = true;
            float ms = 0;
            if ((st = time_steps(b->stream, [&] { return step(trial); }, &ms)) != RR_OK) return st;
            if (ms < bt) {
                bt = ms;
                br = rg;
            }
        }
        for (rr_solver *s : kv.second) {
            s->rows_group = br;
            rr::drop_graph(s);
        }
        b->dirty = true;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_rows_group[kv.first] = br;
    }
    if (steps_run) *steps_run = run;
    return rr_batch_sync(b);
}

} // extern "C"
