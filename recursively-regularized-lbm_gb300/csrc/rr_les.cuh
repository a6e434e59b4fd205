// rr_les.cuh -- the fused time step with the WALE eddy viscosity.
//
// The reference computes tau_t = 3 nu_t from the velocity field of the
// previous step with a 7-point stencil (LES_WALE, LES.cu:4-98) in a launch of
// its own, then collides with tau_eff = tau + tau_t (collision.cu:27-31).
// In the fused step those velocities are the moments this very step computes
// after streaming, so a node needs the moments of its six face neighbours.
//
// Each CTA owns a TX x TY column of nodes and marches over a chunk of z
// planes.  For every plane it computes the moments of the tile plus a
// one-node halo in x and y (no corners: the stencil has none) into a
// three-plane ring of velocity planes in shared memory; the node then takes
// its x/y neighbours from the current plane and its z neighbours from the
// planes before and after.  Halo positions wrap periodically, so partial
// tiles and small domains need no special case; on wall faces the
// reference's one-sided differences never read across the wall.
#pragma once

#include "rr_dispatch.h"
#include "rr_kernels.cuh"

namespace rr {

template <typename S>
struct LesArgs {
    const S *__restrict__ fin;
    S *__restrict__ fout;
    Geom g;
    double tau, cw;
    double F[3];
    int *status;
    int zchunk;
};

__device__ __forceinline__ int wrapn(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

// moments of node (x, y, z) after streaming and walls: velocity into u[]
template <class LT, typename S, typename T, bool FORCE>
__device__ __forceinline__ void node_velocity(const S *__restrict__ fin, const Geom &g, int x, int y,
                                              int z, T Fx, T Fy, T Fz, T (&u)[3]) {
    const uint32_t idx = ((uint32_t)z * (uint32_t)g.ny + (uint32_t)y) * (uint32_t)g.nx + (uint32_t)x;
    T d[LT::Q];
    pull<LT>(fin, g.stride, g.nx, g.ny, g.nz, x, y, z, d);
    if (g.wallmask && any_wall(x, y, z, g)) wall_pass<LT, S, T, FORCE>(fin, g, idx, x, y, z, d, Fx, Fy, Fz);
    Mom<T> m = moments<LT>(d);
    velocity(m, Fx, Fy, Fz, u[0], u[1], u[2]);
}

template <class LT, typename S, bool FORCE>
__global__ void __launch_bounds__(256) les_step_kernel(const LesArgs<S> a) {
    using T = typename CType<S>::T;
    extern __shared__ unsigned char smem_raw[];
    T *us = reinterpret_cast<T *>(smem_raw);
    const Geom &g = a.g;
    const int TX = blockDim.x, TY = blockDim.y;
    const int SX = TX + 2, SY = TY + 2, PL = SX * SY; // one velocity component plane
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * a.zchunk, z1 = min(z0 + a.zchunk, g.nz);
    const T Fx = T(a.F[0]), Fy = T(a.F[1]), Fz = T(a.F[2]);
    const int nhalo = 2 * (TX + TY);

    // fills ring slot `slot` with the velocity of plane z (interior + halo)
    auto plane = [&](int z, int slot) {
        const int zz = wrapn(z, g.nz);
        T *p = us + slot * 3 * PL;
        {
            const int sx = tx + 1, sy = ty + 1;
            T u[3];
            node_velocity<LT, S, T, FORCE>(a.fin, g, wrapn(x0 + tx, g.nx), wrapn(y0 + ty, g.ny), zz, Fx, Fy, Fz, u);
            p[0 * PL + sy * SX + sx] = u[0];
            p[1 * PL + sy * SX + sx] = u[1];
            p[2 * PL + sy * SX + sx] = u[2];
        }
        for (int h = tid; h < nhalo; h += TX * TY) {
            int sx, sy;
            if (h < TY) { sx = 0; sy = h + 1; }
            else if (h < 2 * TY) { sx = TX + 1; sy = h - TY + 1; }
            else if (h < 2 * TY + TX) { sx = h - 2 * TY + 1; sy = 0; }
            else { sx = h - 2 * TY - TX + 1; sy = TY + 1; }
            T u[3];
            node_velocity<LT, S, T, FORCE>(a.fin, g, wrapn(x0 - 1 + sx, g.nx), wrapn(y0 - 1 + sy, g.ny), zz, Fx, Fy, Fz, u);
            p[0 * PL + sy * SX + sx] = u[0];
            p[1 * PL + sy * SX + sx] = u[1];
            p[2 * PL + sy * SX + sx] = u[2];
        }
    };

    const int x = x0 + tx, y = y0 + ty;
    const bool valid = x < g.nx && y < g.ny;
    const bool xlo = g.face[0] != FACE_PERIODIC, xhi = g.face[1] != FACE_PERIODIC;
    const bool ylo = g.face[2] != FACE_PERIODIC, yhi = g.face[3] != FACE_PERIODIC;
    const bool zlo = g.face[4] != FACE_PERIODIC, zhi = g.face[5] != FACE_PERIODIC;
    const T cw = T(a.cw), tau = T(a.tau);

    plane(z0 - 1, 0);
    plane(z0, 1);
    int sm = 0, sc = 1, sp = 2;
#pragma unroll 1
    for (int z = z0; z < z1; z++) {
        plane(z + 1, sp);
        __syncthreads();
        if (valid) {
            const T *pm = us + sm * 3 * PL, *pc = us + sc * 3 * PL, *pp = us + sp * 3 * PL;
            const int c = (ty + 1) * SX + tx + 1;
            T gr[3][3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T *q = pc + k * PL;
                const T uc = q[c];
                // d/dx
                if (x == 0 && xlo) gr[k][0] = (T(3) * uc + q[c + 1]) / T(3);
                else if (x == g.nx - 1 && xhi) gr[k][0] = (T(-3) * uc - q[c - 1]) / T(3);
                else gr[k][0] = T(0.5) * (q[c + 1] - q[c - 1]);
                // d/dy
                if (y == 0 && ylo) gr[k][1] = (T(3) * uc + q[c + SX]) / T(3);
                else if (y == g.ny - 1 && yhi) gr[k][1] = (T(-3) * uc - q[c - SX]) / T(3);
                else gr[k][1] = T(0.5) * (q[c + SX] - q[c - SX]);
                // d/dz
                const T up = pp[k * PL + c], um = pm[k * PL + c];
                if (z == 0 && zlo) gr[k][2] = (T(3) * uc + up) / T(3);
                else if (z == g.nz - 1 && zhi) gr[k][2] = (T(-3) * uc - um) / T(3);
                else gr[k][2] = T(0.5) * (up - um);
            }
            const T taut = wale_tau_t(gr, cw);
            const uint32_t idx = ((uint32_t)z * (uint32_t)g.ny + (uint32_t)y) * (uint32_t)g.nx + (uint32_t)x;
            T d[LT::Q];
            pull<LT>(a.fin, g.stride, g.nx, g.ny, g.nz, x, y, z, d);
            if (g.wallmask && any_wall(x, y, z, g)) wall_pass<LT, S, T, FORCE>(a.fin, g, idx, x, y, z, d, Fx, Fy, Fz);
            Mom<T> m = moments<LT>(d);
            T ux, uy, uz;
            velocity(m, Fx, Fy, Fz, ux, uy, uz);
            if (!(m.drho > T(-0.9) && m.drho < T(9))) atomicOr(a.status, 1);
            const T om1 = T(1) - T(1) / (tau + taut);
            collide<LT, T, FORCE>(d, m, m.drho, ux, uy, uz, om1, Fx, Fy, Fz);
            store_node<LT, S, T>(a.fout, g.stride, idx, d, g.sround != 0, sr_seed(idx, m.drho, ux));
        }
        __syncthreads();
        const int t = sm;
        sm = sc;
        sc = sp;
        sp = t;
    }
}

template <class LT, typename S, bool FORCE>
cudaError_t launch_les_step(const S *fin, S *fout, const Geom &g, double tau, double cw,
                            const double F[3], int *status, const LesTile &tile, cudaStream_t st) {
    using T = typename CType<S>::T;
    LesArgs<S> a;
    a.fin = fin;
    a.fout = fout;
    a.g = g;
    a.tau = tau;
    a.cw = cw;
    a.F[0] = F[0];
    a.F[1] = F[1];
    a.F[2] = F[2];
    a.status = status;
    a.zchunk = tile.zchunk;
    dim3 block(tile.tx, tile.ty, 1);
    dim3 grid((g.nx + tile.tx - 1) / tile.tx, (g.ny + tile.ty - 1) / tile.ty,
              (g.nz + tile.zchunk - 1) / tile.zchunk);
    size_t smem = sizeof(T) * 3 * 3 * (tile.tx + 2) * (tile.ty + 2);
    les_step_kernel<LT, S, FORCE><<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace rr
