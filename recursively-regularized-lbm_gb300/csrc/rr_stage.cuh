// rr_stage.cuh -- the staged DNS step: interior rows through shared memory.
//
// Rows (row = z ny + y) with y in [1, ny-2] and z in [1, nz-2] are taken in
// blocks of R consecutive rows of one z plane.  For population i the R
// source rows of a block, (y0 - cy .. y0 - cy + R - 1, z - cz), are one
// contiguous run of R nx values, so a block needs exactly Q bulk copies
// (cp.async.bulk, global -> shared, completing on an mbarrier).  A persistent
// CTA runs an S-stage pipeline: one thread issues the copies of the block S-1
// ahead while all threads compute the current block from shared memory (the
// x shift of a population is an index offset; a periodic x wraps inside the
// row; a node on an x wall takes its entering populations from its own
// post-collision values, which the producer warp gathers into the stage with
// plain loads after issuing the copies, and applies the closure of that
// face), then store their populations straight to global memory.  Rows on a
// y or z face run in face_kernel, 32 nodes of one row per warp, through the
// wrap-aware pull and the general face loop.  Each node gets the arithmetic
// of the tile step, so the results are the same bit for bit.
//
// Every mbarrier wait is bounded: a wait that gives up (after
// StageArgs::wait_limit polls) sets WATCH_STAGE_WAIT in the watchdog word, the
// CTA stops taking blocks and its issuing thread waits (bounded again, always
// STAGE_WAIT_LIMIT polls) for the copies it still has in flight before it
// exits, so that no bulk copy lands in the shared memory of an exited CTA.
#pragma once

#include "rr_dispatch.h"
#include "rr_kernels.cuh"

namespace rr {

constexpr int STAGE_MAX = 4; // pipeline stages at most

template <int Q, typename S>
struct StageArgs {
    const S *fin;
    S *dst[Q];            // destination of node 0, per population
    Geom g;
    uint32_t nblocks;     // blocks of up to R interior rows
    uint32_t rows;        // R
    uint32_t yblocks;     // blocks per z plane
    FastDiv div_yblocks, div_nxi; // div_nxi: nodes per row in the main loop (nx, or nx - 2 with x walls)
    uint32_t stages;      // S (2 .. STAGE_MAX)
    uint32_t stage_elems; // Q R nx
    double om1;
    double F[3];
    int *status;
    uint32_t wait_limit;  // polls before a pipeline wait gives up (the final drain: STAGE_WAIT_LIMIT)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// true once the phase with parity `parity` has completed; false after `limit`
// unsuccessful polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t k = 0; k < limit; k++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// bytes (a multiple of 16) from global src to shared dst, completing on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// first row and row count of block b
__device__ __forceinline__ void stage_block(uint32_t b, const FastDiv &div_yblocks, uint32_t yblocks, uint32_t R,
                                            int ny, int &z, int &y0, int &rows) {
    const uint32_t zp = fdiv(b, div_yblocks);
    z = 1 + (int)zp;
    y0 = 1 + (int)((b - zp * yblocks) * R);
    rows = min((int)R, ny - 1 - y0);
}

constexpr int STAGE_CONSUMERS = 256;                  // compute threads (8 warps)
constexpr int STAGE_THREADS = STAGE_CONSUMERS + 32;    // + the producer warp

// Warp-specialised pipeline.  Warp 8 (its lane 0) is the producer: for each
// of the CTA's blocks it waits until the 8 compute warps have released the
// stage (empty barrier, one arrive per warp), then issues the block's bulk
// copies onto the stage's full barrier.  The compute warps wait on the full
// barrier, compute, and release the stage; no barrier over the whole CTA.
template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(STAGE_THREADS, 3) stage_kernel(const __grid_constant__ StageArgs<LT::Q, S> a) {
    using T = typename CType<S>::T;
    extern __shared__ __align__(128) unsigned char stage_smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(stage_smem);  // [STAGE_MAX]
    uint64_t *empty = full + STAGE_MAX;                         // [STAGE_MAX]
    S *buf = reinterpret_cast<S *>(stage_smem + 128);
    const Geom &g = a.g;
    const int nx = g.nx;
    const uint32_t NS = a.stages;
    const uint32_t R = a.rows;
    // x walls: the bounce-back sources of the block's x = 0 and x = nx-1 nodes
    // (their own post-collision populations), gathered per stage by the
    // producer warp: wall[s][side][i][r] = f_opp(i) of row r's node on that side
    const bool xwall = g.face[0] != FACE_PERIODIC;
    S *wall = buf + (size_t)NS * a.stage_elems;
    const uint32_t wall_elems = 2u * (uint32_t)LT::Q * R;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < NS; s++) {
            // the copies' expect_tx arrive, plus the gather's arrive with x walls
            mbar_init(&full[s], xwall ? 2 : 1);
            mbar_init(&empty[s], STAGE_CONSUMERS / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // blocks of this CTA: blockIdx.x + k gridDim.x, k = 0 .. mine-1
    const uint32_t mine = blockIdx.x < a.nblocks ? (a.nblocks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (threadIdx.x >= STAGE_CONSUMERS) {
        // the producer warp: lane 0 waits for the stage and issues the bulk
        // copies; with x walls every lane then gathers the wall values (else
        // lane 0 runs alone)
        const uint32_t lane = threadIdx.x & 31u;
        if (!xwall && lane != 0) return;
        const unsigned pmask = xwall ? 0xffffffffu : 1u;
        uint32_t k = 0;
        for (; k < mine; k++) {
            const uint32_t s = k % NS;
            int ok = 1;
            if (lane == 0 && k >= NS && !mbar_wait(&empty[s], (k / NS - 1) & 1u, a.wait_limit)) {
                atomicOr(a.status, WATCH_STAGE_WAIT);
                ok = 0;
            }
            if (!__shfl_sync(pmask, ok, 0)) break;
            int z, y0, rows;
            stage_block(blockIdx.x + k * gridDim.x, a.div_yblocks, a.yblocks, R, g.ny, z, y0, rows);
            if (lane == 0) {
                const uint32_t bytes = (uint32_t)rows * (uint32_t)nx * (uint32_t)sizeof(S);
                S *st = buf + (size_t)s * a.stage_elems;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(&full[s], (uint32_t)LT::Q * bytes);
                static_for<LT::Q>([&](auto ic) {
                    constexpr int i = decltype(ic)::value;
                    const size_t src = (size_t)i * g.stride +
                                       ((size_t)(z - LT::cz(i)) * (size_t)g.ny + (size_t)(y0 - LT::cy(i))) * (size_t)nx;
                    bulk_g2s(st + (size_t)i * R * nx, a.fin + src, bytes, &full[s]);
                });
            }
            if (xwall) {
                S *wb = wall + (size_t)s * wall_elems;
                if ((int)lane < rows) {
                    const uint32_t row0 = ((uint32_t)z * (uint32_t)g.ny + (uint32_t)(y0 + (int)lane)) * (uint32_t)nx;
                    auto gather = [&](auto fc) {
                        constexpr int F = decltype(fc)::value;
                        constexpr uint32_t M = entering_mask<LT, F>();
                        const uint32_t idx = row0 + (F == 0 ? 0u : (uint32_t)nx - 1u);
                        static_for<LT::Q>([&](auto ic) {
                            constexpr int i = decltype(ic)::value;
                            if constexpr (((M >> i) & 1u) != 0)
                                wb[((size_t)F * LT::Q + i) * R + lane] =
                                    a.fin[(unsigned long long)LT::opp(i) * g.stride + idx];
                        });
                    };
                    gather(std::integral_constant<int, 0>{});
                    gather(std::integral_constant<int, 1>{});
                }
                // the warp's stores, then one release arrive for all of them
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
            }
        }
        // before the CTA may leave, every copy it issued has landed (the last
        // use of each stage; bounded)
        if (lane == 0)
            for (uint32_t j = (k > NS ? k - NS : 0); j < k; j++)
                mbar_wait(&full[j % NS], (j / NS) & 1u, STAGE_WAIT_LIMIT);
        return;
    }
    const T Fx = T(a.F[0]), Fy = T(a.F[1]), Fz = T(a.F[2]);
    for (uint32_t k = 0; k < mine; k++) {
        if (!mbar_wait(&full[k % NS], (k / NS) & 1u, a.wait_limit)) {
            if ((threadIdx.x & 31u) == 0) atomicOr(a.status, WATCH_STAGE_WAIT);
            break;
        }
        int z, y0, rows;
        stage_block(blockIdx.x + k * gridDim.x, a.div_yblocks, a.yblocks, R, g.ny, z, y0, rows);
        const S *st = buf + (size_t)(k % NS) * a.stage_elems;
        const S *wb = wall + (size_t)(k % NS) * wall_elems;
        // the main loop takes every node of the block's rows, or with x walls
        // the x in [1, nx-2] ones; the x-wall nodes go to two warps of their own
        const int nxi = xwall ? nx - 2 : nx;
        const int nmain = rows * nxi;
        const int nwall = xwall ? 2 * 32 : 0; // warps 0 and 1 of a second round: x = 0, x = nx - 1
        const int total = ((nmain + STAGE_CONSUMERS - 1) / STAGE_CONSUMERS) * STAGE_CONSUMERS + nwall;
        for (int t = threadIdx.x; t < total; t += STAGE_CONSUMERS) {
            int r, x;
            if (t < nmain) {
                r = (int)fdiv((uint32_t)t, a.div_nxi);
                x = (xwall ? 1 : 0) + t - r * nxi;
            } else {
                const int w = t - (total - nwall);
                if (w < 0) continue;        // padding of the main loop's last round
                r = w & 31;
                if (r >= rows) continue;
                x = w < 32 ? 0 : nx - 1;
            }
            const int y = y0 + r;
            const uint32_t idx = ((uint32_t)z * (uint32_t)g.ny + (uint32_t)y) * (uint32_t)nx + (uint32_t)x;
            const S *row = st + (size_t)r * nx;
            T d[LT::Q];
            if (x >= 1 && x <= nx - 2) {
                static_for<LT::Q>([&](auto ic) {
                    constexpr int i = decltype(ic)::value;
                    d[i] = ld_dev<T>(row + (size_t)i * R * nx + (x - LT::cx(i)));
                });
            } else if (!xwall) {
                // periodic x: the upstream node of an x-face node wraps inside the row
                static_for<LT::Q>([&](auto ic) {
                    constexpr int i = decltype(ic)::value;
                    int xs = x - LT::cx(i);
                    xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
                    d[i] = ld_dev<T>(row + (size_t)i * R * nx + xs);
                });
            } else {
                // an x wall: the entering populations bounce back from this
                // node's own post-collision values (gathered into the stage by
                // the producer), then the face's closure
                auto wallnode = [&](auto fc) {
                    constexpr int F = decltype(fc)::value;
                    constexpr uint32_t M = entering_mask<LT, F>();
                    const T ux = T(g.uw[F][0]), uy = T(g.uw[F][1]), uz = T(g.uw[F][2]);
                    static_for<LT::Q>([&](auto ic) {
                        constexpr int i = decltype(ic)::value;
                        if constexpr (((M >> i) & 1u) != 0) {
                            const T v = ld_dev<T>(wb + ((size_t)F * LT::Q + i) * R + r);
                            d[i] = v + T(6) * (T(LT::cx(i)) * ux + T(LT::cy(i)) * uy + T(LT::cz(i)) * uz);
                        } else {
                            d[i] = ld_dev<T>(row + (size_t)i * R * nx + (x - LT::cx(i)));
                        }
                    });
                    if (g.face[F] == FACE_WALL) regularize<LT, T, FORCE, M>(d, M, Fx, Fy, Fz);
                };
                if (x == 0) wallnode(std::integral_constant<int, 0>{});
                else wallnode(std::integral_constant<int, 1>{});
            }
            Mom<T> m = moments<LT>(d);
            T ux, uy, uz;
            velocity(m, Fx, Fy, Fz, ux, uy, uz);
            if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
            collide<LT, T, FORCE>(d, m, m.drho, ux, uy, uz, T(a.om1), Fx, Fy, Fz);
            if constexpr (std::is_same<S, __half>::value || std::is_same<S, __nv_bfloat16>::value) {
                if (g.sround) {
                    store_sr_pairs<LT, S, T>(d, sr_seed(idx, m.drho, ux), [&](int i) { return a.dst[i] + idx; });
                    continue;
                }
            }
            static_for<LT::Q>([&](auto ic) {
                constexpr int i = decltype(ic)::value;
                st_dev<T>(a.dst[i] + idx, d[i]);
            });
        }
        // this warp is done with stage k % NS
        __syncwarp();
        if ((threadIdx.x & 31u) == 0) mbar_arrive(&empty[k % NS]);
    }
}

// rows on a y or z face (any kind): 32 consecutive nodes of one row per warp
template <int Q, typename S>
struct FaceArgs {
    const S *fin;
    S *dst[Q];
    const S *src[Q]; // upstream addresses of the tile step (single-wall-face nodes)
    Geom g;
    const uint32_t *frows;
    uint32_t nfrows, segs, nitems;
    FastDiv div_segs, div_ny;
    double om1;
    double F[3];
    int *status;
};

template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256, 2) face_kernel(const __grid_constant__ FaceArgs<LT::Q, S> a) {
    using T = typename CType<S>::T;
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (item >= a.nitems) return;
    const Geom &g = a.g;
    const uint32_t r = fdiv(item, a.div_segs);
    const int x = (int)((item - r * a.segs) * 32u + lane);
    if (x >= g.nx) return;
    const uint32_t row = a.frows[r];
    const int z = (int)fdiv(row, a.div_ny);
    const int y = (int)(row - (uint32_t)z * (uint32_t)g.ny);
    const uint32_t idx = row * (uint32_t)g.nx + (uint32_t)x;
    const T Fx = T(a.F[0]), Fy = T(a.F[1]), Fz = T(a.F[2]);
    T d[LT::Q];
    const bool xi = x >= 1 && x <= g.nx - 2, yi = y >= 1 && y <= g.ny - 2, zi = z >= 1 && z <= g.nz - 2;
    const uint32_t faces = g.wallmask & ((x == 0 ? 1u : 0u) | (x == g.nx - 1 ? 2u : 0u) | (y == 0 ? 4u : 0u) |
                                         (y == g.ny - 1 ? 8u : 0u) | (z == 0 ? 16u : 0u) |
                                         (z == g.nz - 1 ? 32u : 0u));
    // one wall face (y or z), interior on the other two axes
    int wf = -1;
    if (faces == 4u || faces == 8u) wf = (xi && zi) ? (faces == 4u ? 2 : 3) : -1;
    else if (faces == 16u || faces == 32u) wf = (xi && yi) ? (faces == 16u ? 4 : 5) : -1;
    switch (wf) {
    case 2: wall_fast<LT, S, T, FORCE, 2>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
    case 3: wall_fast<LT, S, T, FORCE, 3>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
    case 4: wall_fast<LT, S, T, FORCE, 4>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
    case 5: wall_fast<LT, S, T, FORCE, 5>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
    default:
        // as the tile step: the wrap-aware pull, then one face's compiled
        // closure or the general face loop
        pull<LT>(a.fin, g.stride, g.nx, g.ny, g.nz, x, y, z, d);
        if (faces != 0u) {
            if ((faces & (faces - 1u)) == 0u) {
                switch (__ffs(faces) - 1) {
                case 0: wall_face<LT, S, T, FORCE, 0>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                case 1: wall_face<LT, S, T, FORCE, 1>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                case 2: wall_face<LT, S, T, FORCE, 2>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                case 3: wall_face<LT, S, T, FORCE, 3>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                case 4: wall_face<LT, S, T, FORCE, 4>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                default: wall_face<LT, S, T, FORCE, 5>(a.fin, g, idx, d, Fx, Fy, Fz); break;
                }
            } else {
                T tmp[LT::Q];
                static_for<LT::Q>([&](auto ic) {
                    constexpr int i = decltype(ic)::value;
                    tmp[i] = d[i];
                });
                wall_multi<LT, S, T, FORCE>(a.fin, g, idx, x, y, z, Fx, Fy, Fz, tmp);
                static_for<LT::Q>([&](auto ic) {
                    constexpr int i = decltype(ic)::value;
                    d[i] = tmp[i];
                });
            }
        }
        break;
    }
    Mom<T> m = moments<LT>(d);
    T ux, uy, uz;
    velocity(m, Fx, Fy, Fz, ux, uy, uz);
    if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
    collide<LT, T, FORCE>(d, m, m.drho, ux, uy, uz, T(a.om1), Fx, Fy, Fz);
    if constexpr (std::is_same<S, __half>::value || std::is_same<S, __nv_bfloat16>::value) {
        if (g.sround) {
            store_sr_pairs<LT, S, T>(d, sr_seed(idx, m.drho, ux), [&](int i) { return a.dst[i] + idx; });
            return;
        }
    }
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        st_dev<T>(a.dst[i] + idx, d[i]);
    });
}

} // namespace rr
