// rr_aux.cu -- FP64 statistics on the device: the WALE field of a velocity
// readout, diag_flow's domain means and output_profile's y-plane statistics
// (RR27V33_code_DNS_LES/output.cu:24-35 and 181-214), plus the time-averaging
// accumulators.  All reductions have a fixed order (deterministic results).
#include "rr_aux.h"
#include "rr_kernels.cuh"

namespace rr {

// WALE eddy viscosity tau_t = 3 nu_t from FP64 velocity fields (LES.cu:4-98):
// central differences, the reference's one-sided formulas on wall faces.
// Returns 0 where S:S = Sd:Sd = 0 (the reference's 0/0).
__device__ __forceinline__ double wale_tau(const double (&gr)[3][3], double cw) {
    const double dudx = gr[0][0], dudy = gr[0][1], dudz = gr[0][2];
    const double dvdx = gr[1][0], dvdy = gr[1][1], dvdz = gr[1][2];
    const double dwdx = gr[2][0], dwdy = gr[2][1], dwdz = gr[2][2];
    double sijsq = (dudy + dvdx) * (dudy + dvdx) + (dudz + dwdx) * (dudz + dwdx) +
                   (dvdz + dwdy) * (dvdz + dwdy);
    sijsq = 0.5 * sijsq + dudx * dudx + dvdy * dvdy + dwdz * dwdz;
    double s11d = (2. * dudx * dudx - dvdy * dvdy - dwdz * dwdz + dudy * dvdx + dudz * dwdx -
                   2. * dvdz * dwdy) / 3.;
    double s12d = 0.5 * (dudx * (dudy + dvdx) + dudy * dvdy + dvdx * dvdy + dvdz * dwdx + dudz * dwdy);
    double s13d = 0.5 * (dudx * (dudz + dwdx) + dudy * dvdz + dvdx * dwdy + dudz * dwdz + dwdx * dwdz);
    double s22d = (2. * dvdy * dvdy - dudx * dudx - dwdz * dwdz + dudy * dvdx + dvdz * dwdy -
                   2. * dudz * dwdx) / 3.;
    double s23d = 0.5 * (dvdy * (dvdz + dwdy) + dudz * dvdx + dudy * dwdx + dvdz * dwdz + dwdy * dwdz);
    double s33d = (2. * dwdz * dwdz - dudx * dudx - dvdy * dvdy + dudz * dwdx + dvdz * dwdy -
                   2. * dudy * dvdx) / 3.;
    double sd = s11d * s11d + s22d * s22d + s33d * s33d + 2.0 * (s12d * s12d + s13d * s13d + s23d * s23d);
    double den = pow(sijsq, 2.5) + pow(sd, 1.25);
    return den > 0.0 ? 3.0 * cw * cw * pow(sd, 1.5) / den : 0.0;
}

__global__ void __launch_bounds__(256)
wale_kernel(Geom g, double cw, const double *__restrict__ ux, const double *__restrict__ uy,
            const double *__restrict__ uz, double *__restrict__ taut) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n) return;
    int p[3];
    node_xyz(idx, g.nx, g.ny, p[0], p[1], p[2]);
    const int n[3] = {g.nx, g.ny, g.nz};
    const long long st[3] = {1, g.nx, (long long)g.nx * g.ny};
    const double *U[3] = {ux, uy, uz};
    double gr[3][3];
    for (int b = 0; b < 3; b++) {
        const bool lo = g.face[2 * b] != FACE_PERIODIC, hi = g.face[2 * b + 1] != FACE_PERIODIC;
        for (int a2 = 0; a2 < 3; a2++) {
            const double *u = U[a2];
            if (p[b] == 0 && lo) {
                gr[a2][b] = (3.0 * u[idx] + u[idx + st[b]]) / 3.0;
            } else if (p[b] == n[b] - 1 && hi) {
                gr[a2][b] = (-3.0 * u[idx] - u[idx - st[b]]) / 3.0;
            } else {
                long long ip = p[b] == n[b] - 1 ? (long long)idx - (long long)(n[b] - 1) * st[b] : (long long)idx + st[b];
                long long im = p[b] == 0 ? (long long)idx + (long long)(n[b] - 1) * st[b] : (long long)idx - st[b];
                gr[a2][b] = 0.5 * (u[ip] - u[im]);
            }
        }
    }
    taut[idx] = wale_tau(gr, cw);
}

cudaError_t launch_wale(const Geom &g, double cw, const double *ux, const double *uy,
                        const double *uz, double *taut, cudaStream_t st) {
    wale_kernel<<<(g.n + 255) / 256, 256, 0, st>>>(g, cw, ux, uy, uz, taut);
    return cudaGetLastError();
}

// block-wide fixed-order sum of 4 values (256 threads)
__device__ __forceinline__ void block_sum4(double (&v)[4], double (*sh)[256]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; k++) sh[k][t] = v[k];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int k = 0; k < 4; k++) sh[k][t] += sh[k][t + s];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = sh[k][0];
}

// pass 1 of diag_flow's means: per-block partial sums of u, v, w, rho
__global__ void __launch_bounds__(256)
diag_partial_kernel(uint32_t n, const double *__restrict__ ux, const double *__restrict__ uy,
                    const double *__restrict__ uz, const double *__restrict__ rho,
                    double *__restrict__ partial) {
    __shared__ double sh[4][256];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = blockIdx.x * 256u + threadIdx.x; i < n; i += gridDim.x * 256u) {
        v[0] += ux[i];
        v[1] += uy[i];
        v[2] += uz[i];
        v[3] += rho[i];
    }
    block_sum4(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) partial[blockIdx.x * 4 + k] = v[k];
}

// pass 2: one block sums the partials in a fixed order and divides by n
__global__ void __launch_bounds__(256)
diag_final_kernel(int nblocks, uint32_t n, const double *__restrict__ partial, double *__restrict__ out) {
    __shared__ double sh[4][256];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += 256)
        for (int k = 0; k < 4; k++) v[k] += partial[b * 4 + k];
    block_sum4(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) out[k] = v[k] / (double)n;
}

int diag_blocks(uint32_t n) {
    int b = (int)((n + 255u) / 256u);
    return b < DIAG_MAX_BLOCKS ? b : DIAG_MAX_BLOCKS;
}

cudaError_t launch_diag(uint32_t n, const double *ux, const double *uy, const double *uz,
                        const double *rho, double *partial, double *out, cudaStream_t st) {
    const int nb = diag_blocks(n);
    diag_partial_kernel<<<nb, 256, 0, st>>>(n, ux, uy, uz, rho, partial);
    diag_final_kernel<<<1, 256, 0, st>>>(nb, n, partial, out);
    return cudaGetLastError();
}

// one block per y plane: plane means of u, v, w, tau_t, then the second
// moments about those means (output.cu:181-214)
__global__ void __launch_bounds__(256)
profile_kernel(Geom g, double ystar, const double *__restrict__ ux, const double *__restrict__ uy,
               const double *__restrict__ uz, const double *__restrict__ taut,
               double *__restrict__ out) {
    __shared__ double sh[4][256];
    const int iy = blockIdx.x;
    const int cnt = g.nx * g.nz;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < cnt; k += 256) {
        const int ix = k % g.nx, iz = k / g.nx;
        const size_t i = ((size_t)iz * g.ny + iy) * g.nx + ix;
        v[0] += ux[i];
        v[1] += uy[i];
        v[2] += uz[i];
        v[3] += taut ? taut[i] : 0.0;
    }
    block_sum4(v, sh);
    const double mu = v[0] / cnt, mv = v[1] / cnt, mw = v[2] / cnt, mt = v[3] / cnt;
    __syncthreads();
    double a[4] = {0.0, 0.0, 0.0, 0.0}, b[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < cnt; k += 256) {
        const int ix = k % g.nx, iz = k / g.nx;
        const size_t i = ((size_t)iz * g.ny + iy) * g.nx + ix;
        const double ur = ux[i] - mu, vr = uy[i] - mv, wr = uz[i] - mw;
        a[0] += ur * ur;
        a[1] += vr * vr;
        a[2] += wr * wr;
        a[3] += ur * vr;
        b[0] += ur * wr;
        b[1] += vr * wr;
    }
    block_sum4(a, sh);
    __syncthreads();
    block_sum4(b, sh);
    if (threadIdx.x == 0) {
        double *o = out + (size_t)iy * 11;
        o[0] = iy + 0.5;
        o[1] = (iy + 0.5) / ystar;
        o[2] = mu;
        o[3] = mv;
        o[4] = mw;
        o[5] = a[0] / cnt;
        o[6] = a[1] / cnt;
        o[7] = a[2] / cnt;
        o[8] = a[3] / cnt;
        o[9] = b[0] / cnt;
        o[10] = b[1] / cnt;
        out[(size_t)g.ny * 11 + iy] = mt;
    }
}

cudaError_t launch_profile(const Geom &g, double ystar, const double *ux, const double *uy,
                           const double *uz, const double *taut, double *out, cudaStream_t st) {
    profile_kernel<<<g.ny, 256, 0, st>>>(g, ystar, ux, uy, uz, taut, out);
    return cudaGetLastError();
}

__global__ void accumulate_kernel(int m, const double *__restrict__ prof, double *__restrict__ acc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) acc[i] += prof[i];
}

cudaError_t launch_accumulate(int m, const double *prof, double *acc, cudaStream_t st) {
    accumulate_kernel<<<(m + 255) / 256, 256, 0, st>>>(m, prof, acc);
    return cudaGetLastError();
}

// The channel program's start-up trip force of step n (forcing_GP,
// macrovar.cu:76-115) into fx, fy, fz (3 arrays of stride), or the uniform
// force (F0, F1, F2) when trip == 0.  amp = (100 beta / LY) sin(2 pi n / 2000),
// formed on the host; ix / LX is an integer division, as in the reference.
__global__ void __launch_bounds__(256)
trip_force_kernel(double *__restrict__ ff, unsigned long long stride, int LX, int LY, int LZ, int trip,
                  double amp, double phase, double F0, double F1, double F2) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = (uint32_t)LX * (uint32_t)LY * (uint32_t)LZ;
    if (idx >= n) return;
    const int ix = (int)(idx % (uint32_t)LX), iy = (int)((idx / (uint32_t)LX) % (uint32_t)LY),
              iz = (int)(idx / ((uint32_t)LX * (uint32_t)LY));
    double x = F0, y = F1, z = F2;
    if (trip) {
        const double pi2 = 2.0 * 3.14159265358979323846;
        const double LYq = LY / 4;
        const int h0 = 2;
        const double beta9 = 3.0, gamma9 = 2.0;
        y = 0.0;
        z = 0.0;
        if (iy > h0 && iy < LYq + h0) {
            x = F0 * (1.0 - amp * LX / beta9 * sin(pi2 * (iy - h0) / LYq) * sin(beta9 * pi2 * ix / LX) *
                                cos(gamma9 * pi2 * iz / LZ));
            y = F0 * amp * 0.5 * LYq * (1 - cos(pi2 * (iy - h0) / LYq)) * cos(beta9 * pi2 * ix / LX) *
                cos(gamma9 * pi2 * iz / LZ);
            z = F0 * amp * 0.5 * LZ / gamma9 * sin(pi2 * (iy - h0) / LYq) * cos(beta9 * pi2 * ix / LX) *
                sin(gamma9 * pi2 * iz / LZ);
        } else if (iy > 0.75 * LY - h0 && iy < LY - h0) {
            const double ph = (double)(ix / LX) + phase;
            x = F0 * (1.0 + amp * LX / beta9 * sin(pi2 * (-LY + iy + h0 + LYq) / LYq) * sin(beta9 * pi2 * ph) *
                                cos(gamma9 * pi2 * iz / LZ));
            y = -F0 * amp * 0.5 * LYq * (1 - cos(pi2 * (-LY + iy + h0 + LYq) / LYq)) * cos(beta9 * pi2 * ph) *
                cos(gamma9 * pi2 * iz / LZ);
            z = -F0 * amp * 0.5 * LZ / gamma9 * sin(pi2 * (-LY + iy + h0 + LYq) / LYq) * cos(beta9 * pi2 * ph) *
                sin(gamma9 * pi2 * iz / LZ);
        }
    }
    ff[idx] = x;
    ff[stride + idx] = y;
    ff[2 * stride + idx] = z;
}

cudaError_t launch_trip_force(double *ff, unsigned long long stride, int LX, int LY, int LZ, int trip, double amp,
                              double phase, const double F[3], cudaStream_t st) {
    const unsigned long long n = (unsigned long long)LX * LY * LZ;
    trip_force_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ff, stride, LX, LY, LZ, trip, amp, phase, F[0],
                                                                    F[1], F[2]);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
wall_rows_kernel(int nx, int ny, int nz, const double *__restrict__ field, double *__restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t per = (uint32_t)nx * (uint32_t)nz;
    if (t >= 2u * per) return;
    const uint32_t side = t / per, c = t - side * per;
    const uint32_t z = c / (uint32_t)nx, x = c - z * (uint32_t)nx;
    const uint32_t y = side ? (uint32_t)ny - 1u : 0u;
    out[t] = field[(z * (uint32_t)ny + y) * (uint32_t)nx + x];
}

cudaError_t launch_wall_rows(const Geom &g, const double *field, double *out, cudaStream_t st) {
    const uint32_t m = 2u * (uint32_t)g.nx * (uint32_t)g.nz;
    wall_rows_kernel<<<(m + 255) / 256, 256, 0, st>>>(g.nx, g.ny, g.nz, field, out);
    return cudaGetLastError();
}

} // namespace rr
