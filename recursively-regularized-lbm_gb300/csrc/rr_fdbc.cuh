// rr_fdbc.cuh -- the finite-difference wall closure (FDBC, BC.cu:129-309) of
// the y walls, the alternative to the regularized closure that the reference
// ships disabled (main.cu:76-77).
//
// At a wall node (y = 0 or y = ny-1; x and z periodic) FDBC replaces every
// population after streaming:
//   u_w   = 2/3 u(1) - 1/5 u(2)             rows 1 and 2 inward (BC.cu:148-160)
//   S     = strain of u: one-sided second-order d/dy from u_w, u(1), u(2);
//           central d/dx, d/dz from the neighbouring wall nodes' u_w
//   g_i   = feq_i(rho, u_w) + fneq_i(-rho tau_eff S) - Fbar_i feq_i
//   rho   = sum_known f_i / sum_known g_i(rho = 1)   (known: streamed in from
//           inside, BC.cu:243-262)
// then the wall-row moments are taken again (macrovar_BN).  The reference's
// one kernel writes u_w and reads its neighbours' u_w, a race between threads;
// here every u_w of the tile and its one-node halo is formed in shared memory
// first, so each closure reads final values (extrapolate, then close).
//
// The step kernels treat an FDBC face as a bounce-back wall; fdbc_kernel then
// recomputes the wall rows from the same input buffer and overwrites them:
//   MODE 0  DNS step: closure, moments, RR collision, store
//   MODE 1  first WALE pass: closure, moments, velocity into the field u
//   MODE 2  second WALE pass: closure, moments, tau_t from u, collision,
//           store; tau_t of the wall node kept for the next step's closure
//   MODE 3  readout: post-stream populations and FP64 moments
// One CTA of 256 threads per 32 x 8 tile of wall columns, blockIdx.z the face.
#pragma once

#include "rr_kernels.cuh"

namespace rr {

constexpr int FDBC_TX = 32, FDBC_TZ = 8;
constexpr int FDBC_HX = FDBC_TX + 2, FDBC_HZ = FDBC_TZ + 2;
constexpr int FDBC_HALO = FDBC_HX * FDBC_HZ;

template <int Q, typename S>
struct FdbcArgs {
    const S *fin;
    S *fout;
    Geom g;
    double om1, tau, cw;
    double F[3];
    int *status;
    const double *ffp, *ffc;     // per-node forces of the streaming half and the collision (FIELD)
    typename CType<S>::T *u;     // WALE passes: velocity field, 3 arrays of g.stride
    double *wt;                  // WALE: tau_t of the wall nodes, [face][z][x] (NULL for DNS), of
                                 // the collision that wrote fin ...
    double *wt_out;              // ... and of this step's collision (MODE 2)
    double *fo;                  // readout outputs (MODE 3), as readout_kernel
    unsigned long long fo_stride;
    const int *pos;
    double *rho, *ux, *uy, *uz;
    uint32_t faces;              // bit 0: y-lo is FDBC, bit 1: y-hi
};

// 3 CTAs per SM (80 registers): the 384 CTAs of a 384 x 128 channel wall run
// in one wave beside the tile step
template <class LT, typename S, bool FORCE, bool FIELD, int MODE>
__global__ void __launch_bounds__(256, 3) fdbc_kernel(const __grid_constant__ FdbcArgs<LT::Q, S> a) {
    using T = typename CType<S>::T;
    const int side = (int)blockIdx.z;
    if (!((a.faces >> side) & 1u)) return;
    const Geom &g = a.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int x0 = (int)blockIdx.x * FDBC_TX, z0 = (int)blockIdx.y * FDBC_TZ;
    // velocities of rows 1 and 2 inward over the tile and its halo
    __shared__ T us[2][3][FDBC_HALO];
    for (int k = (int)threadIdx.x; k < 2 * FDBC_HALO; k += (int)blockDim.x) {
        const int r = k / FDBC_HALO, c = k - r * FDBC_HALO;
        const int hz = c / FDBC_HX, hx = c - hz * FDBC_HX;
        const int x = (x0 + hx - 1 + nx) % nx, z = (z0 + hz - 1 + nz) % nz;
        const int y = side ? ny - 2 - r : 1 + r;
        const uint32_t idx = ((uint32_t)z * (uint32_t)ny + (uint32_t)y) * (uint32_t)nx + (uint32_t)x;
        T d[LT::Q];
        pull<LT>(a.fin, g.stride, nx, ny, nz, x, y, z, d);
        T Fx, Fy, Fz;
        if constexpr (FIELD) {
            Fx = T(a.ffp[idx]);
            Fy = T(a.ffp[g.stride + idx]);
            Fz = T(a.ffp[2 * g.stride + idx]);
        } else {
            Fx = T(a.F[0]);
            Fy = T(a.F[1]);
            Fz = T(a.F[2]);
        }
        const Mom<T> m = moments<LT>(d);
        T vx, vy, vz;
        velocity(m, Fx, Fy, Fz, vx, vy, vz);
        us[r][0][c] = vx;
        us[r][1][c] = vy;
        us[r][2][c] = vz;
    }
    __syncthreads();
    const int tx = (int)(threadIdx.x & 31u), tz = (int)(threadIdx.x >> 5);
    const int x = x0 + tx, z = z0 + tz;
    if (x >= nx || z >= nz) return;
    const int y = side ? ny - 1 : 0;
    const uint32_t idx = ((uint32_t)z * (uint32_t)ny + (uint32_t)y) * (uint32_t)nx + (uint32_t)x;
    // the extrapolated wall velocity of halo column (hx, hz)
    auto uw = [&](int comp, int hx, int hz) -> T {
        const int c = hz * FDBC_HX + hx;
        return T(2.0 / 3.0) * us[0][comp][c] - T(1.0 / 5.0) * us[1][comp][c];
    };
    const int hx = tx + 1, hz = tz + 1, c0 = hz * FDBC_HX + hx;
    T u0[3], gr[3][3]; // gr[a][b] = d u_a / d x_b
#pragma unroll
    for (int k = 0; k < 3; k++) {
        u0[k] = uw(k, hx, hz);
        const T u1 = us[0][k][c0], u2 = us[1][k][c0];
        gr[k][0] = T(0.5) * (uw(k, hx + 1, hz) - uw(k, hx - 1, hz));
        gr[k][1] = side ? (T(3) * u0[k] - T(4) * u1 + u2) * T(0.5) : (T(-3) * u0[k] + T(4) * u1 - u2) * T(0.5);
        gr[k][2] = T(0.5) * (uw(k, hx, hz + 1) - uw(k, hx, hz - 1));
    }
    const double wt_old = a.wt ? a.wt[((size_t)side * nz + z) * nx + x] : 0.0;
    const T te = T(a.tau + wt_old);
    // -tau_eff S in the order (110, 101, 011, 200, 020, 002)
    T n[6];
    n[0] = -te * (T(0.5) * (gr[0][1] + gr[1][0]));
    n[1] = -te * (T(0.5) * (gr[0][2] + gr[2][0]));
    n[2] = -te * (T(0.5) * (gr[1][2] + gr[2][1]));
    n[3] = -te * gr[0][0];
    n[4] = -te * gr[1][1];
    n[5] = -te * gr[2][2];
    // the force of the streaming half (closure, moments) and, in the modes
    // that collide, of the collision
    T Fx, Fy, Fz, Cx, Cy, Cz;
    if constexpr (FIELD) {
        Fx = T(a.ffp[idx]);
        Fy = T(a.ffp[g.stride + idx]);
        Fz = T(a.ffp[2 * g.stride + idx]);
        if constexpr (MODE == 0 || MODE == 2) {
            Cx = T(a.ffc[idx]);
            Cy = T(a.ffc[g.stride + idx]);
            Cz = T(a.ffc[2 * g.stride + idx]);
        } else {
            Cx = Fx;
            Cy = Fy;
            Cz = Fz;
        }
    } else {
        Fx = Cx = T(a.F[0]);
        Fy = Cy = T(a.F[1]);
        Fz = Cz = T(a.F[2]);
    }
    // g_i(rho = 1) / w_i - 1 for every population
    T Aq[6], Bq[10], Bn[10];
    eq_coeffs(T(1), u0[0], u0[1], u0[2], Aq, Bq);
    third_from_second(n, u0[0], u0[1], u0[2], T(1), Bn);
    const T Fe = FORCE ? T(-1.5) * (u0[0] * Fx + u0[1] * Fy + u0[2] * Fz) : T(0);
    T d[LT::Q];
    T sf = T(0), sg = T(0); // sums over the known populations of w d and w dg
    constexpr double wk = [] {
        double s = 0.0;
        for (int i = 0; i < LT::Q; i++)
            if (LT::cy(i) != 0) s += LT::w(i);
        return s / 2.0; // the populations with c_y < 0 (or > 0): half of those with c_y != 0
    }();
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        const T Ee = even_poly<LT, i>(Aq);
        const T Eo = odd_poly<LT, i>(Bq);
        // fneq = w (sec(a2neq) + thir(a3neq)): twice the half-sums
        T v = Ee + Eo + T(2) * (even_poly<LT, i>(n) + odd_poly<LT, i, T, false>(Bn));
        if constexpr (FORCE) {
            const T Fo = T(1.5) * (T(LT::cx(i)) * Fx + T(LT::cy(i)) * Fy + T(LT::cz(i)) * Fz);
            v -= (T(1) + Ee + Eo) * (Fe + Fo);
        }
        d[i] = v;
        constexpr int cy = LT::cy(i);
        if constexpr (cy != 0) {
            // known: streamed in from the row inside (c_y < 0 at y = 0, > 0 at y = ny-1)
            if ((cy < 0) == (side == 0)) {
                const int xs = (x - LT::cx(i) + nx) % nx, zs = (z - LT::cz(i) + nz) % nz;
                const int ys = y - cy;
                const uint32_t src = ((uint32_t)zs * (uint32_t)ny + (uint32_t)ys) * (uint32_t)nx + (uint32_t)xs;
                const T f = ld_dev<T>(a.fin + (unsigned long long)i * g.stride + src);
                sf += T(LT::w(i)) * f;
                sg += T(LT::w(i)) * v;
            }
        }
    });
    // the density balancing the known populations; g is linear in rho
    const T drho_w = (sf - sg) / (T(wk) + sg);
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        d[i] = d[i] + drho_w * (T(1) + d[i]);
    });
    if constexpr (MODE == 3) {
        readout_node<LT, T>(d, idx, false, FIELD ? a.ffp[idx] : a.F[0], FIELD ? a.ffp[g.stride + idx] : a.F[1],
                            FIELD ? a.ffp[2 * g.stride + idx] : a.F[2], a.fo, a.fo_stride, a.pos, a.rho, a.ux,
                            a.uy, a.uz);
        return;
    }
    const Mom<T> m = moments<LT>(d);
    T vx, vy, vz;
    velocity(m, Fx, Fy, Fz, vx, vy, vz);
    if constexpr (MODE == 1) {
        a.u[idx] = vx;
        a.u[g.stride + idx] = vy;
        a.u[2ull * g.stride + idx] = vz;
        return;
    }
    if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
    T om1 = T(a.om1);
    if constexpr (MODE == 2) {
        const T tt = les_taut<T>(a.u, g, x, y, z, idx, T(a.cw));
        om1 = T(1) - T(1) / (T(a.tau) + tt);
        a.wt_out[((size_t)side * nz + z) * nx + x] = double(tt);
    }
    collide<LT, T, FORCE>(d, m, m.drho, vx, vy, vz, om1, Cx, Cy, Cz);
    store_node<LT, S, T>(a.fout, g.stride, idx, d, g.sround != 0, sr_seed(idx, m.drho, vx));
}

} // namespace rr
