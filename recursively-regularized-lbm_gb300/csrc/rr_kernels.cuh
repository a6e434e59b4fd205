// rr_kernels.cuh -- the fused RR-LBM time step and its companions.
//
// State in HBM: one array per population ("SoA"), f_i of node
// (x, y, z) at fin[i * stride + (z * ny + y) * nx + x], stored as the
// deviation d_i = f_i / w_i - 1 in FP64, FP32, FP16 or BF16.  Two such arrays
// ping-pong: a step reads the post-collision state of the previous step and
// writes its own.
//
// One step (one launch) per node, in the reference's order (main.cu:360-409):
//   pull-stream from the neighbours with periodic wrap  (streaming.cu:3-24)
//   wall faces x-lo, x-hi, y-lo, y-hi, z-lo, z-hi in that order:
//     half-way bounce-back with moving-wall term         (BB, streaming.cu:26-56;
//                                                         Cavity/streaming.f90:91-152)
//     regularized closure of the entering populations    (RRBC, BC.cu:4-126)
//   moments rho, u = (sum c f + F/2) / rho               (macrovar.cu:4-31)
//   [WALE eddy viscosity from the neighbours' velocities] (LES.cu:4-98)
//   RR collision                                         (collision.cu:4-120)
// The reference runs the collision first and the streaming last; the fused
// kernel runs the same sequence shifted by half a step, so its state is the
// post-collision one.  The macroscopic fields the reference holds after step
// n are produced on demand by readout_kernel (pull + walls + moments from the
// previous buffer).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rr_node.cuh"
#include "rr_pair.cuh"

namespace rr {

// FACE_FDBC: bounce-back inside the step kernels, then the wall rows are
// rebuilt by fdbc_kernel (rr_fdbc.cuh)
enum FaceKind : int { FACE_PERIODIC = 0, FACE_WALL = 1, FACE_WALL_BB = 2, FACE_FDBC = 3 };

struct Geom {
    int nx, ny, nz;
    uint32_t n;          // nodes
    unsigned long long stride; // elements between population arrays (>= n)
    int face[6];         // FaceKind of x-lo, x-hi, y-lo, y-hi, z-lo, z-hi
    double uw[6][3];     // wall velocity of each face
    uint32_t wallmask;   // bit f: face f is a wall
    int sround;          // FP16/BF16 storage: stochastic (1) or nearest (0) rounding
    int bgk;             // BGK collision with the incompressible velocity (else RR)
    uint32_t fdbc;       // y rows left to fdbc_kernel by the tile step: bit 0 y = 0, bit 1 y = ny-1
};

template <typename S> struct CType { using T = float; };
template <> struct CType<double> { using T = double; };

template <typename T> __device__ __forceinline__ T ld_dev(const double *p) { return T(*p); }
template <typename T> __device__ __forceinline__ T ld_dev(const float *p) { return T(*p); }
template <typename T> __device__ __forceinline__ T ld_dev(const __half *p) { return T(__half2float(*p)); }
template <typename T> __device__ __forceinline__ T ld_dev(const __nv_bfloat16 *p) {
    return T(__bfloat162float(*p));
}
template <typename T> __device__ __forceinline__ void st_dev(double *p, T v) { *p = double(v); }
template <typename T> __device__ __forceinline__ void st_dev(float *p, T v) { *p = float(v); }
template <typename T> __device__ __forceinline__ void st_dev(__half *p, T v) { *p = __float2half_rn(float(v)); }
template <typename T> __device__ __forceinline__ void st_dev(__nv_bfloat16 *p, T v) {
    *p = __float2bfloat16_rn(float(v));
}

// 32-bit integer finaliser (xor-shift / multiply), used as a counter-free
// source of rounding noise
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Stochastic rounding to 16 bits rounds a value up in magnitude with
// probability (dropped fraction) / (unit in the last place), so the stored
// value is unbiased.  Round-to-nearest stalls a slowly varying field whose
// per-step change is below half a unit in the last place (e.g. the Ma = 0.01
// Taylor-Green decay); unbiased rounding keeps that change in expectation.
// Two FP32 values to a 16-bit pair with the hardware's stochastic rounding
// (cvt.rs, sm_100-family): hi goes to bits 31:16, lo to bits 15:0, rbits
// supplies the random bits.
template <typename S>
__device__ __forceinline__ uint32_t cvt_sr2(float hi, float lo, uint32_t rbits) {
    uint32_t h2;
    if constexpr (std::is_same<S, __half>::value)
        asm("cvt.rs.satfinite.f16x2.f32 %0, %1, %2, %3;" : "=r"(h2) : "f"(hi), "f"(lo), "r"(rbits));
    else
        asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(h2) : "f"(hi), "f"(lo), "r"(rbits));
    return h2;
}

// Stochastic-rounding store of one node's populations to FP16/BF16, two
// populations per conversion.  The random bits: one hash of the node seeds a
// linear-congruential stream, one 32-bit draw per pair, folded as
// r ^ (r >> 16) so that both halves carry high-order LCG bits.  at(i) is the
// address of population i.
template <class LT, typename S, typename T, class Addr>
__device__ __forceinline__ void store_sr_pairs(const T (&d)[LT::Q], uint32_t seed, Addr at) {
    uint32_t r = seed;
    static_for<(LT::Q + 1) / 2>([&](auto jc) {
        constexpr int i0 = 2 * decltype(jc)::value, i1 = i0 + 1;
        r = r * 1664525u + 1013904223u;
        float v1 = 0.0f;
        if constexpr (i1 < LT::Q) v1 = float(d[i1]);
        const uint32_t h2 = cvt_sr2<S>(v1, float(d[i0]), r ^ (r >> 16));
        *reinterpret_cast<unsigned short *>(at(i0)) = (unsigned short)(h2 & 0xFFFFu);
        if constexpr (i1 < LT::Q) *reinterpret_cast<unsigned short *>(at(i1)) = (unsigned short)(h2 >> 16);
    });
}

// seed of a node's rounding stream: its index and its post-collision density
// and velocity (so that it changes from step to step)
template <typename T>
__device__ __forceinline__ uint32_t sr_seed(uint32_t idx, T drho, T ux) {
    return mix32(idx * 0x9E3779B9u ^ __float_as_uint(float(drho)) ^ (__float_as_uint(float(ux)) * 0x85EBCA6Bu));
}

// store a node's post-collision populations, coalesced across the warp
template <class LT, typename S, typename T>
__device__ __forceinline__ void store_node(S *__restrict__ fout, unsigned long long stride, uint32_t idx,
                                           const T (&d)[LT::Q], bool sround, uint32_t seed) {
    if constexpr (std::is_same<S, __half>::value || std::is_same<S, __nv_bfloat16>::value) {
        if (sround) {
            store_sr_pairs<LT, S, T>(d, seed, [&](int i) { return fout + (unsigned long long)i * stride + idx; });
            return;
        }
    }
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        st_dev<T>(fout + (unsigned long long)i * stride + idx, d[i]);
    });
}

__device__ __forceinline__ void node_xyz(uint32_t idx, int nx, int ny, int &x, int &y, int &z) {
    uint32_t t = idx / (uint32_t)nx;
    x = (int)(idx - t * (uint32_t)nx);
    z = (int)(t / (uint32_t)ny);
    y = (int)(t - (uint32_t)z * (uint32_t)ny);
}

// pull every population from its upstream neighbour, periodic wrap on all axes
// (walls overwrite the wrapped values afterwards, as in the reference)
template <class LT, typename S, typename T>
__device__ __forceinline__ void pull(const S *__restrict__ fin, unsigned long long stride, int nx,
                                     int ny, int nz, int x, int y, int z, T (&d)[LT::Q]) {
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const int zm = z == 0 ? nz - 1 : z - 1, zp = z == nz - 1 ? 0 : z + 1;
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        constexpr int cx = LT::cx(i), cy = LT::cy(i), cz = LT::cz(i);
        const int xs = cx > 0 ? xm : (cx < 0 ? xp : x);
        const int ys = cy > 0 ? ym : (cy < 0 ? yp : y);
        const int zs = cz > 0 ? zm : (cz < 0 ? zp : z);
        const uint32_t src = ((uint32_t)zs * (uint32_t)ny + (uint32_t)ys) * (uint32_t)nx + (uint32_t)xs;
        d[i] = ld_dev<T>(fin + (unsigned long long)i * stride + src);
    });
}

__device__ __forceinline__ bool on_face(int f, int x, int y, int z, const Geom &g) {
    switch (f) {
    case 0: return x == 0;
    case 1: return x == g.nx - 1;
    case 2: return y == 0;
    case 3: return y == g.ny - 1;
    case 4: return z == 0;
    default: return z == g.nz - 1;
    }
}

__device__ __forceinline__ bool any_wall(int x, int y, int z, const Geom &g) {
    const uint32_t m = g.wallmask;
    return ((m & 1u) && x == 0) || ((m & 2u) && x == g.nx - 1) || ((m & 4u) && y == 0) ||
           ((m & 8u) && y == g.ny - 1) || ((m & 16u) && z == 0) || ((m & 32u) && z == g.nz - 1);
}

// wall faces in the reference order: bounce-back from the post-collision
// opposite population of this node plus 6 c_i.U_wall (in deviation form
// d_i = d*_ibar + 6 c_i.U), then the regularized closure of the same
// populations when the face is FACE_WALL
template <class LT, typename S, typename T, bool FORCE>
__device__ __forceinline__ void wall_pass(const S *__restrict__ fin, const Geom &g, uint32_t idx, int x,
                                       int y, int z, T (&d)[LT::Q], T Fx, T Fy, T Fz) {
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        if (!((g.wallmask >> f) & 1u) || !on_face(f, x, y, z, g)) continue;
        const int axis = f >> 1;
        const bool hi = f & 1;
        const T ux = T(g.uw[f][0]), uy = T(g.uw[f][1]), uz = T(g.uw[f][2]);
        uint32_t mask = 0;
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr int o = LT::opp(i);
            const int c = axis == 0 ? LT::cx(i) : (axis == 1 ? LT::cy(i) : LT::cz(i));
            const bool ent = hi ? (c < 0) : (c > 0);
            if (ent) {
                mask |= 1u << i;
                T v = ld_dev<T>(fin + (unsigned long long)o * g.stride + idx);
                d[i] = v + T(6) * (T(LT::cx(i)) * ux + T(LT::cy(i)) * uy + T(LT::cz(i)) * uz);
            }
        });
        if (g.face[f] == FACE_WALL) regularize<LT, T, FORCE>(d, mask, Fx, Fy, Fz);
    }
}

// General step over an explicit list of nodes (any node: wrap-aware pull and
// the wall faces).  Used for grids too thin for the tile kernel (nx < 3).
template <typename S>
struct StepArgs {
    const S *__restrict__ fin;
    S *__restrict__ fout;
    Geom g;
    double om1;       // 1 - 1/tau
    double F[3];      // uniform body force
    int *status;      // watchdog flag (bit 0: density out of range / NaN)
    uint32_t count;   // nodes of this launch
    const uint32_t *__restrict__ list; // node indices
};

// DNS step: one thread per node
template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256) step_kernel(const StepArgs<S> a) {
    using T = typename CType<S>::T;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.count) return;
    int x, y, z;
    const uint32_t idx = a.list[t];
    node_xyz(idx, a.g.nx, a.g.ny, x, y, z);
    T d[LT::Q];
    pull<LT>(a.fin, a.g.stride, a.g.nx, a.g.ny, a.g.nz, x, y, z, d);
    const T Fx = T(a.F[0]), Fy = T(a.F[1]), Fz = T(a.F[2]);
    if (a.g.wallmask && any_wall(x, y, z, a.g)) wall_pass<LT, S, T, FORCE>(a.fin, a.g, idx, x, y, z, d, Fx, Fy, Fz);
    Mom<T> m = moments<LT>(d);
    T ux, uy, uz;
    velocity(m, Fx, Fy, Fz, ux, uy, uz);
    if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
    collide<LT, T, FORCE>(d, m, m.drho, ux, uy, uz, T(a.om1), Fx, Fy, Fz);
    store_node<LT, S, T>(a.fout, a.g.stride, idx, d, a.g.sround != 0, sr_seed(idx, m.drho, ux));
}

// Division by a run-time constant d < 2^31 for numerators n < 2^31:
// q = (umulhi(n, m) + n) >> s with s = ceil(log2 d), m = 2^32 (2^s - d) / d + 1.
struct FastDiv {
    uint32_t d, m, s;
};
__host__ inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t s = 0;
    while ((1ull << s) < d) s++;
    const unsigned long long m = ((1ull << 32) * ((1ull << s) - d)) / d + 1;
    return FastDiv{d, (uint32_t)m, s};
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
    return (__umulhi(n, f.m) + n) >> f.s;
}

// One-launch step with warp-granular work items.  The grid's warps walk
// groups of rows_group x-rows (row = z*ny + y; rows_group a multiple of 32,
// picked per size class by the autotuner).  A group holds, per row,
// ceil((nx-2)/32) items of 32 consecutive nodes over x in [1, nx-2], and then
// 2 rows_group / 32 items with the x = 0 and the x = nx-1 nodes of its rows,
// 32 rows per item.  The x-face nodes are therefore processed in the same
// window as their rows (the data they need sits in L2), they fill whole CTAs
// of their own (a slow warp does not hold a CTA of fast ones resident), and
// every item is uniform over its warp: rows off every y/z face take the fast
// path (no wrap, no wall, precomputed population addresses); wall /
// periodic-edge rows and x-face items take the wrap-aware pull and, per node,
// the closure of its wall face compiled for that face (edge and corner
// nodes: the general face loop, out of line).

template <int Q, typename S>
struct TileArgs {
    const S *src[Q]; // fast path: upstream-neighbour address of node 0, per population
    S *dst[Q];       // destination of node 0, per population
    const S *fin;
    Geom g;
    uint32_t nitems, nrows, segs, group_items;
    uint32_t pairs;                  // row items take 64 nodes, two x-adjacent nodes per lane (packed FP32 pairs)
    uint32_t rows_group, xf_half;    // rows per group; x-face items per face per group
    uint32_t nmain;                  // items of the row groups; the rest are edge items
    const uint32_t *edges;           // x-end nodes of rows on a y/z wall face
    uint32_t nedges;
    uint32_t yzwall;                 // bit 0: y-lo, 1: y-hi, 2: z-lo, 3: z-hi walls
    uint32_t rot;                    // row rotation: (nz-1)*ny puts the last z plane first
    FastDiv div_group, div_segs, div_ny, div_nx;
    double om1;
    double F[3];
    int *status;
    typename CType<S>::T *u; // WALE passes: velocity field, 3 arrays of g.stride
    double tau, cw;          // WALE collide pass: molecular tau, C_w
    // per-node force fields (3 arrays of g.stride each; FIELD instantiations):
    // ffp for the streaming half of the step (walls, moments), ffc for the
    // collision
    const double *ffp, *ffc;
};

// populations entering the domain through face F (0..5 = x-lo .. z-hi)
template <class LT, int F>
__host__ __device__ constexpr uint32_t entering_mask() {
    uint32_t m = 0;
    for (int i = 0; i < LT::Q; i++) {
        const int c = F / 2 == 0 ? LT::cx(i) : (F / 2 == 1 ? LT::cy(i) : LT::cz(i));
        if ((F & 1) ? c < 0 : c > 0) m |= 1u << i;
    }
    return m;
}

// one wall face known at compile time: bounce-back + regularized closure of
// its entering populations only
template <class LT, typename S, typename T, bool FORCE, int F>
__device__ __forceinline__ void wall_face(const S *__restrict__ fin, const Geom &g, uint32_t idx, T (&d)[LT::Q],
                                          T Fx, T Fy, T Fz) {
    constexpr uint32_t M = entering_mask<LT, F>();
    const T ux = T(g.uw[F][0]), uy = T(g.uw[F][1]), uz = T(g.uw[F][2]);
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        if constexpr (((M >> i) & 1u) != 0) {
            constexpr int o = LT::opp(i);
            const T v = ld_dev<T>(fin + (unsigned long long)o * g.stride + idx);
            d[i] = v + T(6) * (T(LT::cx(i)) * ux + T(LT::cy(i)) * uy + T(LT::cz(i)) * uz);
        }
    });
    if (g.face[F] == FACE_WALL) regularize<LT, T, FORCE, M>(d, M, Fx, Fy, Fz);
}

// A node on exactly one wall face F and at least one node away from every
// other face: its populations that do not enter through F come from inside
// the domain (no wrap), so they use the fast path's precomputed addresses;
// the entering ones are bounced back from this node's own post-collision
// populations.  Then the regularized closure of the entering set.
template <class LT, typename S, typename T, bool FORCE, int F>
__device__ __forceinline__ void wall_fast(const S *const *src, const S *__restrict__ fin, const Geom &g,
                                          uint32_t idx, T (&d)[LT::Q], T Fx, T Fy, T Fz) {
    constexpr uint32_t M = entering_mask<LT, F>();
    const T ux = T(g.uw[F][0]), uy = T(g.uw[F][1]), uz = T(g.uw[F][2]);
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        if constexpr (((M >> i) & 1u) != 0) {
            constexpr int o = LT::opp(i);
            const T v = ld_dev<T>(fin + (unsigned long long)o * g.stride + idx);
            d[i] = v + T(6) * (T(LT::cx(i)) * ux + T(LT::cy(i)) * uy + T(LT::cz(i)) * uz);
        } else {
            d[i] = ld_dev<T>(src[i] + idx);
        }
    });
    if (g.face[F] == FACE_WALL) regularize<LT, T, FORCE, M>(d, M, Fx, Fy, Fz);
}

// nodes on two or three wall faces (edges and corners of a walled box): the
// face loop in the reference order, out of line (rare)
template <class LT, typename S, typename T, bool FORCE>
__device__ __noinline__ void wall_multi(const S *__restrict__ fin, const Geom &g, uint32_t idx, int x, int y,
                                        int z, T Fx, T Fy, T Fz, T *dd) {
    T d[LT::Q];
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        d[i] = dd[i];
    });
    wall_pass<LT, S, T, FORCE>(fin, g, idx, x, y, z, d, Fx, Fy, Fz);
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        dd[i] = d[i];
    });
}

// resident CTAs per SM the tile step is compiled for (register budget 65536 /
// (256 x that)).  The packed-pair form of the DNS step (PAIRS: two nodes'
// populations live per thread) runs FP16/BF16 at 3 CTAs, 80 registers (at 2
// CTAs, 128 registers, 2 % slower), FP32 and the forced step at 2 (FP32
// pairs take twice the registers for their loads; the forced collision at 80
// registers spills: channel 0.44 ms per step against 0.355 at 2 CTAs).  One node per thread: the force-free DNS step at 5
// (48 registers), the forced one and the trip-forcing step at 4, the WALE
// passes and the BGK step at 5.
#ifndef RR_WALE_MIN_BLOCKS
#define RR_WALE_MIN_BLOCKS 5
#endif
template <typename S, bool FORCE = false> __host__ __device__ constexpr int pair_min_blocks() {
    return (sizeof(S) == 2 && !FORCE) ? 3 : 2;
}
template <typename S, bool FORCE = false, int MODE = 0, bool FIELD = false, bool BGK = false, bool PAIRS = false>
constexpr int tile_min_blocks() {
    return sizeof(S) == 8 ? 2
           : PAIRS        ? pair_min_blocks<S, FORCE>()
           : MODE != 0    ? RR_WALE_MIN_BLOCKS
           : FIELD        ? 4
           : BGK          ? 5
           : FORCE        ? 4
                          : 5;
}
// the batch kernel holds its loop state and the shared descriptor on top of
// the tile step's registers
template <typename S, bool FORCE = false> constexpr int batch_min_blocks() {
    return sizeof(S) == 8 ? 2 : pair_min_blocks<S, FORCE>();
}

template <typename T> __device__ __forceinline__ T rr_sqrt(T v);
template <> __device__ __forceinline__ float rr_sqrt(float v) { return sqrtf(v); }
template <> __device__ __forceinline__ double rr_sqrt(double v) { return sqrt(v); }

// WALE tau_t of LES.cu:79-97 from the velocity gradient g[a][b] = du_a/dx_b.
// x^1.5, x^2.5 and x^1.25 are formed from square roots; S:S = Sd:Sd = 0 gives 0
// where the reference gives 0/0.
template <typename T>
__device__ __forceinline__ T wale_tau_t(const T (&gr)[3][3], T cw) {
    const T dudx = gr[0][0], dudy = gr[0][1], dudz = gr[0][2];
    const T dvdx = gr[1][0], dvdy = gr[1][1], dvdz = gr[1][2];
    const T dwdx = gr[2][0], dwdy = gr[2][1], dwdz = gr[2][2];
    T sijsq = (dudy + dvdx) * (dudy + dvdx) + (dudz + dwdx) * (dudz + dwdx) + (dvdz + dwdy) * (dvdz + dwdy);
    sijsq = T(0.5) * sijsq + dudx * dudx + dvdy * dvdy + dwdz * dwdz;
    const T third = T(1) / T(3);
    T s11d = (T(2) * dudx * dudx - dvdy * dvdy - dwdz * dwdz + dudy * dvdx + dudz * dwdx - T(2) * dvdz * dwdy) * third;
    T s12d = T(0.5) * (dudx * (dudy + dvdx) + dudy * dvdy + dvdx * dvdy + dvdz * dwdx + dudz * dwdy);
    T s13d = T(0.5) * (dudx * (dudz + dwdx) + dudy * dvdz + dvdx * dwdy + dudz * dwdz + dwdx * dwdz);
    T s22d = (T(2) * dvdy * dvdy - dudx * dudx - dwdz * dwdz + dudy * dvdx + dvdz * dwdy - T(2) * dudz * dwdx) * third;
    T s23d = T(0.5) * (dvdy * (dvdz + dwdy) + dudz * dvdx + dudy * dwdx + dvdz * dwdz + dwdy * dwdz);
    T s33d = (T(2) * dwdz * dwdz - dudx * dudx - dvdy * dvdy + dudz * dwdx + dvdz * dwdy - T(2) * dudy * dvdx) * third;
    T sd = s11d * s11d + s22d * s22d + s33d * s33d + T(2) * (s12d * s12d + s13d * s13d + s23d * s23d);
    const T rs = rr_sqrt(sijsq), rd = rr_sqrt(sd);
    const T den = sijsq * sijsq * rs + sd * rr_sqrt(rd); // S:S^2.5 + Sd:Sd^1.25
    return den > T(0) ? T(3) * cw * cw * (sd * rd) / den : T(0);
}

// tau_t of node (x, y, z) from the velocity field u (3 arrays of g.stride):
// central differences with periodic wrap, the reference's one-sided
// differences (3 u0 + u1) / 3 and (-3 u_{N-1} - u_{N-2}) / 3 on wall faces
// (LES.cu:20-78)
template <typename T>
__device__ __forceinline__ T les_taut(const T *__restrict__ u, const Geom &g, int x, int y, int z, uint32_t idx,
                                      T cw) {
    const uint32_t nx = (uint32_t)g.nx, nxy = (uint32_t)g.nx * (uint32_t)g.ny;
    const uint32_t ixm = x == 0 ? idx + nx - 1u : idx - 1u;
    const uint32_t ixp = x == g.nx - 1 ? idx - (nx - 1u) : idx + 1u;
    const uint32_t iym = y == 0 ? idx + (uint32_t)(g.ny - 1) * nx : idx - nx;
    const uint32_t iyp = y == g.ny - 1 ? idx - (uint32_t)(g.ny - 1) * nx : idx + nx;
    const uint32_t izm = z == 0 ? idx + (uint32_t)(g.nz - 1) * nxy : idx - nxy;
    const uint32_t izp = z == g.nz - 1 ? idx - (uint32_t)(g.nz - 1) * nxy : idx + nxy;
    const bool xlo = x == 0 && g.face[0] != FACE_PERIODIC, xhi = x == g.nx - 1 && g.face[1] != FACE_PERIODIC;
    const bool ylo = y == 0 && g.face[2] != FACE_PERIODIC, yhi = y == g.ny - 1 && g.face[3] != FACE_PERIODIC;
    const bool zlo = z == 0 && g.face[4] != FACE_PERIODIC, zhi = z == g.nz - 1 && g.face[5] != FACE_PERIODIC;
    T gr[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const T *q = u + (unsigned long long)k * g.stride;
        const T uc = q[idx];
        const T xm = q[ixm], xp = q[ixp], ym = q[iym], yp = q[iyp], zm = q[izm], zp = q[izp];
        gr[k][0] = xlo ? (T(3) * uc + xp) / T(3) : (xhi ? (T(-3) * uc - xm) / T(3) : T(0.5) * (xp - xm));
        gr[k][1] = ylo ? (T(3) * uc + yp) / T(3) : (yhi ? (T(-3) * uc - ym) / T(3) : T(0.5) * (yp - ym));
        gr[k][2] = zlo ? (T(3) * uc + zp) / T(3) : (zhi ? (T(-3) * uc - zm) / T(3) : T(0.5) * (zp - zm));
    }
    return wale_tau_t(gr, cw);
}

// BGK single-relaxation-time collision of the BGK program (BGK/collision.cu:
// 11-33) in deviation form d = f / w - 1: feq / w = rho + p with
// p = eu + (eu^2 - uv) / 2, eu = 3 c.u, uv = 3 u.u, so
// d* = d - (d - (drho + p)) / tau + (1 - 1 / (2 tau)) 3 (c.F - u.F) (1 + p)
template <class LT, typename T, bool FORCE>
__host__ __device__ __forceinline__ void collide_bgk(T (&d)[LT::Q], T drho, T ux, T uy, T uz, T inv_tau, T Fx,
                                                     T Fy, T Fz) {
    const T uv = T(3) * (ux * ux + uy * uy + uz * uz);
    const T kf = T(1) - T(0.5) * inv_tau;
    const T uF = ux * Fx + uy * Fy + uz * Fz;
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        constexpr int cx = LT::cx(i), cy = LT::cy(i), cz = LT::cz(i);
        const T eu = T(3) * (T(cx) * ux + T(cy) * uy + T(cz) * uz);
        const T p = eu + T(0.5) * (eu * eu - uv);
        T v = d[i] - (d[i] - (drho + p)) * inv_tau;
        if constexpr (FORCE) v += kf * T(3) * (T(cx) * Fx + T(cy) * Fy + T(cz) * Fz - uF) * (T(1) + p);
        d[i] = v;
    });
}

// one node of the tile step (row, x, y, z); fast: a row off every y/z face and
// x in [1, nx-2] (no wrap, no wall: the precomputed upstream addresses)
template <class LT, typename S, bool FORCE, int MODE, bool FIELD, bool BGK, class A>
__device__ __forceinline__ void tile_node(const A &a, uint32_t row, int x, int y, int z, bool fast) {
    using T = typename CType<S>::T;
    const Geom &g = a.g;
    // the finite-difference closure's wall rows: fdbc_kernel writes them
    if (!fast && g.fdbc && (((g.fdbc & 1u) && y == 0) || ((g.fdbc & 2u) && y == g.ny - 1))) return;
    const uint32_t idx = row * (uint32_t)g.nx + (uint32_t)x;
    // the force of the streaming half (walls, moments) and of the collision
    T Fx, Fy, Fz, Cx, Cy, Cz;
    if constexpr (FIELD) {
        Fx = T(a.ffp[idx]);
        Fy = T(a.ffp[g.stride + idx]);
        Fz = T(a.ffp[2 * g.stride + idx]);
        Cx = T(a.ffc[idx]);
        Cy = T(a.ffc[g.stride + idx]);
        Cz = T(a.ffc[2 * g.stride + idx]);
    } else {
        Fx = Cx = T(a.F[0]);
        Fy = Cy = T(a.F[1]);
        Fz = Cz = T(a.F[2]);
    }
    T d[LT::Q];
    if (fast) {
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            d[i] = ld_dev<T>(a.src[i] + idx);
        });
    } else {
        const bool xi = x >= 1 && x <= g.nx - 2, yi = y >= 1 && y <= g.ny - 2, zi = z >= 1 && z <= g.nz - 2;
        const uint32_t faces = g.wallmask & ((x == 0 ? 1u : 0u) | (x == g.nx - 1 ? 2u : 0u) | (y == 0 ? 4u : 0u) |
                                             (y == g.ny - 1 ? 8u : 0u) | (z == 0 ? 16u : 0u) |
                                             (z == g.nz - 1 ? 32u : 0u));
        // one wall face, interior on the other two axes
        int wf = -1;
        if (faces == 1u || faces == 2u) wf = (yi && zi) ? (faces == 1u ? 0 : 1) : -1;
        else if (faces == 4u || faces == 8u) wf = (xi && zi) ? (faces == 4u ? 2 : 3) : -1;
        else if (faces == 16u || faces == 32u) wf = (xi && yi) ? (faces == 16u ? 4 : 5) : -1;
        switch (wf) {
        case 0: wall_fast<LT, S, T, FORCE, 0>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        case 1: wall_fast<LT, S, T, FORCE, 1>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        case 2: wall_fast<LT, S, T, FORCE, 2>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        case 3: wall_fast<LT, S, T, FORCE, 3>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        case 4: wall_fast<LT, S, T, FORCE, 4>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        case 5: wall_fast<LT, S, T, FORCE, 5>(a.src, a.fin, g, idx, d, Fx, Fy, Fz); break;
        default: break;
        }
        if (wf < 0) pull<LT>(a.fin, g.stride, g.nx, g.ny, g.nz, x, y, z, d);
        if (wf < 0 && faces != 0u) {
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
    }
    Mom<T> m = moments<LT>(d);
    T ux, uy, uz;
    if constexpr (BGK) {
        // BGK/macrovar.cu:27-29: u = sum c f + F/2
        ux = m.jx + T(0.5) * Fx;
        uy = m.jy + T(0.5) * Fy;
        uz = m.jz + T(0.5) * Fz;
    } else {
        velocity(m, Fx, Fy, Fz, ux, uy, uz);
    }
    if constexpr (MODE == 1) {
        a.u[idx] = ux;
        a.u[g.stride + idx] = uy;
        a.u[2ull * g.stride + idx] = uz;
        return;
    }
    if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
    T om1 = T(a.om1);
    if constexpr (MODE == 2) om1 = T(1) - T(1) / (T(a.tau) + les_taut<T>(a.u, g, x, y, z, idx, T(a.cw)));
    if constexpr (BGK) collide_bgk<LT, T, FORCE>(d, m.drho, ux, uy, uz, T(1) - om1, Cx, Cy, Cz);
    else collide<LT, T, FORCE>(d, m, m.drho, ux, uy, uz, om1, Cx, Cy, Cz);
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

// Stores the populations of two x-adjacent nodes ia, ia + 1 (ia even): one
// aligned word per population (32 bits for FP16/BF16, 64 for FP32), whole
// sectors across the warp; keep (put_word) drops a node that another work
// item owns.  With stochastic rounding each node draws from its own stream
// exactly as store_sr_pairs does for a node alone: per population pair
// (i0, i1) one LCG draw r, folded f = r ^ (r >> 16), whose low half rounds i0
// and high half i1; one packed conversion rounds population i of both nodes,
// the first node's bits in the low half of the random operand, the second's
// in the high.
template <class LT, typename S, bool PARTIAL = false>
__device__ __forceinline__ void store_pair(S *const *dst, uint32_t ia, const F2 (&d)[LT::Q], bool sround,
                                           uint32_t sa, uint32_t sb, uint32_t keep = 3u) {
    // keep: 3 both nodes, 0 neither; PARTIAL also 1 / 2 (one node: one more
    // store instruction per population for the whole warp)
    auto put = [&](S *p, typename PairWord<S>::W w) {
        if constexpr (PARTIAL) put_word<S>(p, w, keep);
        else if (keep != 0u) *reinterpret_cast<typename PairWord<S>::W *>(p) = w;
    };
    if constexpr (std::is_same<S, __half>::value || std::is_same<S, __nv_bfloat16>::value) {
        if (sround) {
            uint32_t ra = sa, rb = sb;
            static_for<(LT::Q + 1) / 2>([&](auto jc) {
                constexpr int i0 = 2 * decltype(jc)::value, i1 = i0 + 1;
                ra = ra * 1664525u + 1013904223u;
                rb = rb * 1664525u + 1013904223u;
                const uint32_t fa = ra ^ (ra >> 16), fb = rb ^ (rb >> 16);
                put(dst[i0] + ia, cvt_sr2<S>(d[i0].hi(), d[i0].lo(), __byte_perm(fa, fb, 0x5410)));
                if constexpr (i1 < LT::Q) put(dst[i1] + ia, cvt_sr2<S>(d[i1].hi(), d[i1].lo(), __byte_perm(fa, fb, 0x7632)));
            });
            return;
        }
    }
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        put(dst[i] + ia, word_of<S>(d[i]));
    });
}

// the DNS step of the node pair ia, ia + 1 from its post-stream populations
// d: moments, the watchdog, the collision, the stores (keep: 3 both nodes, 0
// neither: the pair belongs to another item)
template <class LT, typename S, bool FORCE>
__device__ __forceinline__ void pair_core(F2 (&d)[LT::Q], uint32_t ia, S *const *dst, double om1_, const double *Fv,
                                          int *status, bool sround, uint32_t keep) {
    const F2 Fx(Fv[0]), Fy(Fv[1]), Fz(Fv[2]);
    Mom<F2> m = moments<LT>(d);
    F2 ux, uy, uz;
    velocity(m, Fx, Fy, Fz, ux, uy, uz);
    const bool ok_lo = m.drho.lo() > -0.9f && m.drho.lo() < 9.0f, ok_hi = m.drho.hi() > -0.9f && m.drho.hi() < 9.0f;
    if (((keep & 1u) && !ok_lo) || ((keep & 2u) && !ok_hi)) atomicOr(status, 1);
    collide<LT, F2, FORCE>(d, m, m.drho, ux, uy, uz, F2(om1_), Fx, Fy, Fz);
    store_pair<LT, S>(dst, ia, d, sround, sr_seed(ia, m.drho.lo(), ux.lo()), sr_seed(ia + 1u, m.drho.hi(), ux.hi()),
                      keep);
}

// Two x-adjacent nodes x, x + 1 (x even) of a row off every y/z face.  The
// warp holds the 64-node segment [x0, x0 + 64) of the row (x0 a multiple of
// 64; lanes past the row's end load nothing and store nothing).  Each
// population is one aligned word load from its upstream row, whole sectors
// across the warp; a population with c_x = +1 takes the element below its
// word from the lane below by a shuffle, c_x = -1 the element above from the
// lane above, and the segment's first (c_x = +1) and last (c_x = -1) lane load
// their missing element alone, wrapped periodically in x.  Every lane of the
// warp must call this (the shuffles take all 32).  The pair is collided in
// packed FP32 (pair_core), bit for bit the scalar node arithmetic.  xends:
// x walls, whose end pairs (0, 1) and (nx-2, nx-1) belong to the x-face items
// (xend_pair); the lanes holding them only feed their neighbours' shuffles.
template <class LT, typename S, bool FORCE, class A>
__device__ __forceinline__ void pair_row(const A &a, uint32_t row, int x0, uint32_t lane, bool xends) {
    using W = typename PairWord<S>::W;
    const Geom &g = a.g;
    const int nx = g.nx;
    const int x = x0 + 2 * (int)lane;
    const bool active = x < nx;
    const uint32_t rbase = row * (uint32_t)nx;
    const bool last = active && (x + 2 >= nx || lane == 31u);
    const int xlo = x0 == 0 ? nx - 1 : x0 - 1; // the first lane's element at x - 1
    const int xhi = x + 2 >= nx ? 0 : x + 2;   // the last lane's element at x + 2
    F2 d[LT::Q];
    if constexpr (sizeof(S) == 4) {
        // FP32 words (64 bits): every load first (the words and the end
        // lanes' missing elements), then the shuffles, so that all loads are
        // in flight together (interleaved, the shuffles held them back:
        // cavity 128^3 153 us against 100 us per step)
        W w[LT::Q], e[LT::Q];
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr int cx = LT::cx(i);
            // element 0 of the upstream row of population i
            const S *up = a.src[i] + (rbase + (uint32_t)cx);
            w[i] = active ? ld_word<S>(up + x) : W(0);
            if constexpr (cx == 1) e[i] = lane == 0u ? elem_hi<S>(up + xlo) : W(0);
            if constexpr (cx == -1) e[i] = last ? elem_lo<S>(up + xhi) : W(0);
        });
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr int cx = LT::cx(i);
            W v = w[i];
            if constexpr (cx == 1) {
                const W b = __shfl_up_sync(0xFFFFFFFFu, v, 1);
                v = join_word<S>(lane == 0u ? e[i] : b, v);
            } else if constexpr (cx == -1) {
                const W b = __shfl_down_sync(0xFFFFFFFFu, v, 1);
                v = join_word<S>(v, last ? e[i] : b);
            }
            d[i] = word_f2<S>(v);
        });
    } else {
        // 16-bit words: population by population (loads first measured
        // Taylor-Green 128^3 65 against 60 us per step)
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr int cx = LT::cx(i);
            // element 0 of the upstream row of population i
            const S *up = a.src[i] + (rbase + (uint32_t)cx);
            W w = active ? ld_word<S>(up + x) : W(0);
            if constexpr (cx == 1) {
                W b = __shfl_up_sync(0xFFFFFFFFu, w, 1);
                if (lane == 0u) b = elem_hi<S>(up + xlo);
                w = join_word<S>(b, w);
            } else if constexpr (cx == -1) {
                W b = __shfl_down_sync(0xFFFFFFFFu, w, 1);
                if (last) b = elem_lo<S>(up + xhi);
                w = join_word<S>(w, b);
            }
            d[i] = word_f2<S>(w);
        });
    }
    if (!active) return;
    const uint32_t keep = xends && (x == 0 || x + 2 == nx) ? 0u : 3u;
    pair_core<LT, S, FORCE>(d, rbase + (uint32_t)x, a.dst, a.om1, a.F, a.status, g.sround != 0, keep);
}

// The end pair of a row off every y/z face with x walls, in an x-face item
// (one row per lane): LO the pair (0, 1), else (nx-2, nx-1).  The words of
// the pair from the upstream rows, the inner node's shifted element alone;
// the wall node's entering populations bounce back with that face's closure
// in scalar FP32 (wall_face, as the node alone gets it); then both nodes
// collide as a packed pair and store whole words.
template <class LT, typename S, bool FORCE, bool LO, class A>
__device__ __forceinline__ void xend_pair(const A &a, uint32_t row) {
    using W = typename PairWord<S>::W;
    const Geom &g = a.g;
    const int nx = g.nx;
    const uint32_t rbase = row * (uint32_t)nx;
    const int x = LO ? 0 : nx - 2;
    const uint32_t idx = rbase + (uint32_t)x;
    W v[LT::Q];
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        constexpr int cx = LT::cx(i);
        const S *up = a.src[i] + (rbase + (uint32_t)cx);
        W w = ld_word<S>(up + x);
        // the wall node's entering element (0 here) is replaced below
        if constexpr (cx == 1) w = join_word<S>(LO ? W(0) : elem_hi<S>(up + (x - 1)), w);
        if constexpr (cx == -1) w = join_word<S>(w, LO ? elem_lo<S>(up + (x + 2)) : W(0));
        v[i] = w;
    });
    float t[LT::Q];
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        t[i] = LO ? word_f2<S>(v[i]).lo() : word_f2<S>(v[i]).hi();
    });
    const float Fx = float(a.F[0]), Fy = float(a.F[1]), Fz = float(a.F[2]);
    if constexpr (LO) wall_face<LT, S, float, FORCE, 0>(a.fin, g, idx, t, Fx, Fy, Fz);
    else wall_face<LT, S, float, FORCE, 1>(a.fin, g, idx + 1u, t, Fx, Fy, Fz);
    F2 d[LT::Q];
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        const F2 w = word_f2<S>(v[i]);
        d[i] = LO ? F2(t[i], w.hi()) : F2(w.lo(), t[i]);
    });
    pair_core<LT, S, FORCE>(d, idx, a.dst, a.om1, a.F, a.status, g.sround != 0, 3u);
}

// A row item of the aligned pair layout, a 64-node segment of one row: false
// for the other items (x-face and edge items, the one-node path's).  Without
// x walls the segments cover every x and there are no other items; with x
// walls the x = 0 and x = nx-1 nodes stay with the x-face and edge items.  A
// row on a y/z face or a periodic edge row takes the general node path, each
// lane its two nodes one after the other.
template <class LT, typename S, bool FORCE, class A>
__device__ __forceinline__ bool pair_item(const A &a, uint32_t item, uint32_t lane) {
    if (item >= a.nitems) return true; // the whole warp: nothing
    const Geom &g = a.g;
    const uint32_t nedge_items = a.nitems - a.nmain;
    if (item < nedge_items) return false;
    const uint32_t mitem = item - nedge_items;
    const uint32_t grp = fdiv(mitem, a.div_group);
    const uint32_t sub = mitem - grp * a.group_items;
    if (sub >= a.rows_group * a.segs) return false;
    const uint32_t rl = fdiv(sub, a.div_segs);
    uint32_t row = grp * a.rows_group + rl;
    if (row >= a.nrows) return true; // the whole warp: nothing
    row += a.rot;
    if (row >= a.nrows) row -= a.nrows;
    const int z = (int)fdiv(row, a.div_ny);
    const int y = (int)(row - (uint32_t)z * (uint32_t)g.ny);
    const int x0 = (int)(sub - rl * a.segs) * 64;
    const bool xends = a.xf_half != 0;
    if (y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2) {
        pair_row<LT, S, FORCE>(a, row, x0, lane, xends);
        return true;
    }
    const int x = x0 + 2 * (int)lane;
    if (x >= g.nx) return true;
#pragma unroll 1
    for (int k = 0; k < 2; k++)
        if (!xends || (x + k != 0 && x + k != g.nx - 1))
            tile_node<LT, S, FORCE, 0, false, false>(a, row, x + k, y, z, false);
    return true;
}

// The node a lane of work item `item` takes in the one-node layout: false if
// none.  The slow items go first so that they overlap the bulk instead of
// forming a tail: the edge items, then the rows of the last z plane (the row
// order is rotated by one plane).
template <class A>
__device__ __forceinline__ bool tile_decode(const A &a, uint32_t item, uint32_t lane, uint32_t &row, int &x, int &y,
                                            int &z, bool &fast) {
    if (item >= a.nitems) return false;
    const Geom &g = a.g;
    const uint32_t nedge_items = a.nitems - a.nmain;
    if (item >= nedge_items) {
        const uint32_t mitem = item - nedge_items;
        const uint32_t grp = fdiv(mitem, a.div_group);
        const uint32_t sub = mitem - grp * a.group_items;
        bool xface = false;
        if (sub < a.rows_group * a.segs) {
            const uint32_t rl = fdiv(sub, a.div_segs);
            row = grp * a.rows_group + rl;
            x = 1 + (int)((sub - rl * a.segs) * 32u + lane);
            fast = true;
            if (x > g.nx - 2) return false;
        } else {
            // the x = 0 nodes of the group's rows, 32 per item, then the
            // x = nx-1 nodes: whole CTAs of these slower items
            const uint32_t xi = sub - a.rows_group * a.segs;
            const bool lo = xi < a.xf_half;
            row = grp * a.rows_group + (lo ? xi : xi - a.xf_half) * 32u + lane;
            x = lo ? 0 : g.nx - 1;
            fast = false;
            xface = true;
        }
        if (row >= a.nrows) return false;
        row += a.rot;
        if (row >= a.nrows) row -= a.nrows;
        z = (int)fdiv(row, a.div_ny);
        y = (int)(row - (uint32_t)z * (uint32_t)g.ny);
        const bool yzw = ((a.yzwall & 1u) && y == 0) || ((a.yzwall & 2u) && y == g.ny - 1) ||
                         ((a.yzwall & 4u) && z == 0) || ((a.yzwall & 8u) && z == g.nz - 1);
        if (xface && yzw) return false; // an edge node: handled by the edge items
        fast = fast && y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2;
    } else {
        const uint32_t e = item * 32u + lane;
        if (e >= a.nedges) return false;
        const uint32_t nidx = a.edges[e];
        row = fdiv(nidx, a.div_nx);
        x = (int)(nidx - row * (uint32_t)g.nx);
        z = (int)fdiv(row, a.div_ny);
        y = (int)(row - (uint32_t)z * (uint32_t)g.ny);
        fast = false;
    }
    return true;
}

// one work item (one warp) of the tile step; A is TileArgs wherever it lives
// (kernel parameters for one domain, shared memory for a batch).  MODE 0: the
// DNS step.  The WALE step is two passes over the same items: MODE 1 streams,
// applies the walls and writes the velocity field; MODE 2 streams again,
// takes tau_t from the 7-point stencil of that field and collides.
template <class LT, typename S, bool FORCE, int MODE = 0, bool FIELD = false, bool BGK = false, bool PAIRS = true,
          class A>
__device__ __forceinline__ void tile_item(const A &a, uint32_t item, uint32_t lane) {
    // the aligned pair layout: 16- and 32-bit storage, the DNS step with a
    // uniform force and the RR collision (the host sets a.pairs only then,
    // and only for an even nx); PAIRS = false compiles it out
    constexpr bool PAIRABLE = PAIRS && sizeof(S) <= 4 && MODE == 0 && !FIELD && !BGK;
    if constexpr (PAIRABLE) {
        if (a.pairs && pair_item<LT, S, FORCE>(a, item, lane)) return;
    }
    uint32_t row;
    int x, y, z;
    bool fast;
    if (!tile_decode(a, item, lane, row, x, y, z, fast)) return;
    if constexpr (PAIRABLE) {
        // pair layout: an x-face node of a row off every y/z face takes its
        // end pair
        if (a.pairs && y >= 1 && y <= a.g.ny - 2 && z >= 1 && z <= a.g.nz - 2) {
            if (x == 0) xend_pair<LT, S, FORCE, true>(a, row);
            else xend_pair<LT, S, FORCE, false>(a, row);
            return;
        }
    }
    tile_node<LT, S, FORCE, MODE, FIELD, BGK>(a, row, x, y, z, fast);
}

// PAIRS: the DNS step in the packed-pair layout (a.pairs set); else one node
// per lane, compiled for more resident CTAs
template <class LT, typename S, bool FORCE, int MODE = 0, bool FIELD = false, bool BGK = false, bool PAIRS = false>
__global__ void __launch_bounds__(256, tile_min_blocks<S, FORCE, MODE, FIELD, BGK, PAIRS>())
    tile_kernel(const __grid_constant__ TileArgs<LT::Q, S> a) {
    tile_item<LT, S, FORCE, MODE, FIELD, BGK, PAIRS>(a, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                                                     threadIdx.x & 31u);
}


// Many domains in one persistent launch.  The CTAs of every domain's tile
// step (blockDim / 32 items each) are numbered consecutively, domain after
// domain (cta_begin: prefix sums; cta_dom: the domain of every CTA); the
// persistent grid walks them either strided (CTA t of the grid takes t,
// t + grid, ...) or in contiguous chunks.  A CTA copies the descriptor of the
// domain it enters into shared memory and runs the same work items as that
// domain's own tile launch, so every node of a domain gets the arithmetic
// (and rounding stream) it gets alone.  The domain of the next CTA is read by
// every thread (one broadcast load), so the threads agree without a barrier;
// barriers are taken only around a descriptor change.
template <int Q, typename S>
struct BatchArgs {
    const TileArgs<Q, S> *desc; // per domain, for this step's buffer parity
    const uint32_t *cta_begin;  // [ndom + 1]
    const uint32_t *cta_dom;    // [total_ctas]
    uint32_t ndom, total_ctas;
    uint32_t chunk;             // 0: strided walk; else CTAs per persistent CTA
};

template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256, batch_min_blocks<S, FORCE>()) batch_kernel(const __grid_constant__ BatchArgs<LT::Q, S> b) {
    using TA = TileArgs<LT::Q, S>;
    static_assert(sizeof(TA) % 8 == 0, "descriptor copy is by 8-byte words");
    __shared__ __align__(16) unsigned long long sdesc[sizeof(TA) / 8];
    const TA &a = *reinterpret_cast<const TA *>(sdesc);
    const uint32_t wpc = blockDim.x >> 5; // items per CTA
    uint32_t t, end, inc;
    if (b.chunk) {
        t = blockIdx.x * b.chunk;
        end = min(t + b.chunk, b.total_ctas);
        inc = 1;
    } else {
        t = blockIdx.x;
        end = b.total_ctas;
        inc = gridDim.x;
    }
    uint32_t cur = 0xFFFFFFFFu, first = 0;
    for (; t < end; t += inc) {
        const uint32_t dom = __ldg(b.cta_dom + t);
        if (dom != cur) {
            if (cur != 0xFFFFFFFFu) __syncthreads(); // every warp is done with the old descriptor
            const unsigned long long *src = reinterpret_cast<const unsigned long long *>(b.desc + dom);
            for (uint32_t w = threadIdx.x; w < sizeof(TA) / 8; w += blockDim.x) sdesc[w] = __ldg(src + w);
            __syncthreads();
            cur = dom;
            first = __ldg(b.cta_begin + dom);
        }
        tile_item<LT, S, FORCE>(a, (t - first) * wpc + (threadIdx.x >> 5), threadIdx.x & 31u);
    }
}

// 1 / r to within a few units of the last FP64 place: the FP32 reciprocal
// refined by one Newton-Raphson step x' = x (2 - r x), which squares its
// relative error (~6e-8 -> ~4e-15)
__device__ __forceinline__ double recip_nr(double r) {
    const double x = double(1.0f / float(r));
    return x * fma(-r, x, 2.0);
}

// a readout's outputs of one node from its post-stream deviations d.
// ACC selects the moment arithmetic:
//   0: FP64 per population, w_i (1 + d_i) summed (macrovar.cu:18-28), for FP64 storage;
//   1: FP64 sums of d_i per weight class k = |c_i|^2, rho = 1 + sum_k w_k s_k,
//      j = sum_k w_k (signed class sums), for 32-bit storage (the same sums,
//      reassociated: the w_i of opposite populations cancel exactly);
//   2: as 1 with the class sums in FP32 and rho - 1, j, u in FP32, for 16-bit
//      storage, whose values FP32 holds exactly (11 or 8 significant bits): the
//      FP32 rounding of the sums (~1e-7 relative) is far below the storage's.
// FP64 throughput on this part is a small fraction of FP32: modes 1 and 2 keep the
// readout of a narrow state memory-bound.
template <class LT, typename T, int ACC = 0>
__device__ __forceinline__ void readout_node(const T (&d)[LT::Q], uint32_t idx, bool bgk, double Fx_, double Fy_,
                                             double Fz_, double *__restrict__ fo, unsigned long long fo_stride,
                                             const int *__restrict__ pos, double *__restrict__ rho,
                                             double *__restrict__ ux_o, double *__restrict__ uy_o,
                                             double *__restrict__ uz_o) {
    if (fo) {
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            fo[(unsigned long long)pos[i] * fo_stride + idx] = LT::w(i) * (1.0 + double(d[i]));
        });
    }
    if constexpr (ACC != 0) {
        if (!rho) return;
        using A = typename std::conditional<ACC == 2, float, double>::type;
        A s[4] = {}, sx[4] = {}, sy[4] = {}, sz[4] = {};
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr int k = LT::nnz(i);
            const A v = A(d[i]);
            s[k] += v;
            if constexpr (LT::cx(i) > 0) sx[k] += v;
            if constexpr (LT::cx(i) < 0) sx[k] -= v;
            if constexpr (LT::cy(i) > 0) sy[k] += v;
            if constexpr (LT::cy(i) < 0) sy[k] -= v;
            if constexpr (LT::cz(i) > 0) sz[k] += v;
            if constexpr (LT::cz(i) < 0) sz[k] -= v;
        });
        constexpr int NK = LT::Q == 27 ? 4 : 3;
        A dr = A(LT::Set::weight_of(0)) * s[0], jx = 0, jy = 0, jz = 0;
#pragma unroll
        for (int k = 1; k < NK; k++) {
            const A wk = A(LT::Set::weight_of(k));
            dr += wk * s[k];
            jx += wk * sx[k];
            jy += wk * sy[k];
            jz += wk * sz[k];
        }
        const double r = 1.0 + double(dr);
        rho[idx] = r;
        jx += A(0.5 * Fx_);
        jy += A(0.5 * Fy_);
        jz += A(0.5 * Fz_);
        if (bgk) { // the incompressible velocity, not divided by rho
            ux_o[idx] = double(jx);
            uy_o[idx] = double(jy);
            uz_o[idx] = double(jz);
        } else if constexpr (ACC == 2) {
            const float ri = 1.0f / (1.0f + float(dr));
            ux_o[idx] = double(jx * ri);
            uy_o[idx] = double(jy * ri);
            uz_o[idx] = double(jz * ri);
        } else {
            const double ri = recip_nr(r);
            ux_o[idx] = jx * ri;
            uy_o[idx] = jy * ri;
            uz_o[idx] = jz * ri;
        }
        return;
    }
    if (rho) {
        // moments in FP64 from the stored state (macrovar.cu:18-28)
        double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const double fv = LT::w(i) * (1.0 + double(d[i]));
            r += fv;
            if constexpr (LT::cx(i) > 0) jx += fv;
            if constexpr (LT::cx(i) < 0) jx -= fv;
            if constexpr (LT::cy(i) > 0) jy += fv;
            if constexpr (LT::cy(i) < 0) jy -= fv;
            if constexpr (LT::cz(i) > 0) jz += fv;
            if constexpr (LT::cz(i) < 0) jz -= fv;
        });
        rho[idx] = r;
        // BGK: the incompressible velocity, not divided by rho
        ux_o[idx] = bgk ? jx + 0.5 * Fx_ : (jx + 0.5 * Fx_) / r;
        uy_o[idx] = bgk ? jy + 0.5 * Fy_ : (jy + 0.5 * Fy_) / r;
        uz_o[idx] = bgk ? jz + 0.5 * Fz_ : (jz + 0.5 * Fz_) / r;
    }
}

// Readout: the reference's post-stream state after the last step, from the
// previous post-collision buffer.  Writes FP64 f (reference layout, ordering
// given by pos: internal population i goes to output population pos[i]) and/or the
// macroscopic fields.  The boundary nodes' general wall path runs out of line
// (wall_multi): inlined, it set the register count for every node (158
// registers, one CTA per SM; a 128^3 FP16 readout took 0.4 ms).
template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256, sizeof(S) == 8 ? 2 : 4)
readout_kernel(const S *__restrict__ fin, Geom g, double Fx_, double Fy_, double Fz_,
               double *__restrict__ fo, unsigned long long fo_stride, const int *__restrict__ pos,
               double *__restrict__ rho, double *__restrict__ ux_o, double *__restrict__ uy_o,
               double *__restrict__ uz_o, const double *__restrict__ ff) {
    using T = typename CType<S>::T;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n) return;
    if (ff) { // a per-node force field: 3 arrays of g.stride
        Fx_ = ff[idx];
        Fy_ = ff[g.stride + idx];
        Fz_ = ff[2 * g.stride + idx];
    }
    int x, y, z;
    node_xyz(idx, g.nx, g.ny, x, y, z);
    T d[LT::Q];
    pull<LT>(fin, g.stride, g.nx, g.ny, g.nz, x, y, z, d);
    const T Fx = T(Fx_), Fy = T(Fy_), Fz = T(Fz_);
    if (g.wallmask && any_wall(x, y, z, g)) {
        // the general face loop, out of line (its registers stay off the
        // interior nodes' path)
        T tmp[LT::Q];
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            tmp[i] = d[i];
        });
        wall_multi<LT, S, T, FORCE>(fin, g, idx, x, y, z, Fx, Fy, Fz, tmp);
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            d[i] = tmp[i];
        });
    }
    readout_node<LT, T, sizeof(S) == 8 ? 0 : sizeof(S) == 4 ? 1 : 2>(d, idx, g.bgk != 0, Fx_, Fy_, Fz_, fo,
                                                                      fo_stride, pos, rho, ux_o, uy_o, uz_o);
}

// State upload: populations in the reference's post-stream form (FP64,
// reference layout; internal population i is input population pos[i]) plus the macroscopic fields the first
// collision is to use (init_arrays, initial.cu:268-326, stores macros that
// are not the moments of f).  Collides and writes the post-collision state.
template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256)
upload_kernel(S *__restrict__ fout, Geom g, double tau, double omc, double Fx_, double Fy_, double Fz_,
              const double *__restrict__ fi, unsigned long long fi_stride, const int *__restrict__ pos,
              const double *__restrict__ rho, const double *__restrict__ ux,
              const double *__restrict__ uy, const double *__restrict__ uz,
              const double *__restrict__ taut, const double *__restrict__ ff) {
    using T = typename CType<S>::T;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n) return;
    if (ff) { // a per-node force field: 3 arrays of g.stride
        Fx_ = ff[idx];
        Fy_ = ff[g.stride + idx];
        Fz_ = ff[2 * g.stride + idx];
    }
    T d[LT::Q];
    if (fi) {
        // internal population i is input population pos[i]
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            d[i] = T(fi[(unsigned long long)pos[i] * fi_stride + idx] / LT::w(i) - 1.0);
        });
    } else if constexpr (sizeof(S) < 8) {
        // the equilibrium below in FP32 arithmetic for 16/32-bit storage (the
        // result is rounded to the storage type; FP64 throughput is a small
        // fraction of FP32 on this part)
        const float dr = float(rho[idx] - 1.0), r = float(rho[idx]);
        const float u0 = float(ux[idx]), u1 = float(uy[idx]), u2 = float(uz[idx]);
        const float uv = 3.0f * (u0 * u0 + u1 * u1 + u2 * u2);
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const float eu = 3.0f * (float(LT::cx(i)) * u0 + float(LT::cy(i)) * u1 + float(LT::cz(i)) * u2);
            d[i] = dr + r * (eu + 0.5f * (eu * eu - uv));
        });
    } else {
        // second-order equilibrium of (rho, u), Cavity/collision.f90:103-114:
        // feq = w rho (1 + eu + (eu^2 - uv)/2), eu = c.u / cs^2, uv = u.u / cs^2
        const double r = rho[idx], u0 = ux[idx], u1 = uy[idx], u2 = uz[idx];
        const double uv = 3.0 * (u0 * u0 + u1 * u1 + u2 * u2);
        static_for<LT::Q>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const double eu = 3.0 * (LT::cx(i) * u0 + LT::cy(i) * u1 + LT::cz(i) * u2);
            d[i] = T((r - 1.0) + r * (eu + 0.5 * (eu * eu - uv)));
        });
    }
    Mom<T> m = moments<LT>(d);
    // relaxation factor (BGK 1 / tau, RR 1 - 1 / tau): the host's omc unless
    // tau_t varies per node
    const double om = !taut ? omc : g.bgk ? 1.0 / (tau + taut[idx]) : 1.0 - 1.0 / (tau + taut[idx]);
    if (g.bgk)
        collide_bgk<LT, T, FORCE>(d, T(rho[idx] - 1.0), T(ux[idx]), T(uy[idx]), T(uz[idx]), T(om), T(Fx_), T(Fy_),
                                  T(Fz_));
    else
        collide<LT, T, FORCE>(d, m, T(rho[idx] - 1.0), T(ux[idx]), T(uy[idx]), T(uz[idx]), T(om), T(Fx_), T(Fy_),
                              T(Fz_));
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        st_dev<T>(fout + (unsigned long long)i * g.stride + idx, d[i]);
    });
}

} // namespace rr
