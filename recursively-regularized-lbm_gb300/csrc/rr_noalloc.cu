// rr_noalloc.cu -- diag_flow's domain means without any device allocation.
//
// rr_diag() reduces through partial sums in memory the solver allocated.
// Some callers cannot allocate device memory at the moment they want the
// statistics: a server that has handed its whole HBM budget to resident
// domains (admission control counts every byte, so a statistics call may not
// take more), or a latency-critical loop in which a cudaMalloc -- which can
// synchronise the device -- is not acceptable.  rr_diag_fields_noalloc()
// serves them: the caller passes the FP64 fields (already on the device) and a
// device output, and the partial sums live in a fixed array reserved when the
// library is loaded.
//
// The scratch array below is static device memory: every GPU on which the
// library is loaded holds it (32 KiB) until the process exits.  In host code
// its name is a host-side stand-in, not a device address, so the kernels get
// its device address from cudaGetSymbolAddress, looked up once per device
// (with that device current) by the first call on that device.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "rr_api.h"

namespace {

constexpr int NOALLOC_BLOCKS = 1024; // partial-sum blocks: 1024 x 4 doubles = 32 KiB
constexpr int NOALLOC_THREADS = 256;
constexpr int MAX_DEVICES = 64;

// Shared by every call on a device and keeping the last call's contents.
// Each call's first pass writes every slot its second pass reads, so nothing
// has to be cleared between calls; two calls that overlap on the GPU (on
// different streams, or from different host threads) race on this array.
__device__ __align__(256) double g_diag_scratch[4 * NOALLOC_BLOCKS];

double *g_scratch_addr[MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mutex;

__device__ __forceinline__ void sum4(double (&v)[4], double (*sh)[NOALLOC_THREADS]) {
    const int t = threadIdx.x;
    for (int k = 0; k < 4; k++) sh[k][t] = v[k];
    __syncthreads();
    for (int s = NOALLOC_THREADS / 2; s > 0; s >>= 1) {
        if (t < s)
            for (int k = 0; k < 4; k++) sh[k][t] += sh[k][t + s];
        __syncthreads();
    }
    for (int k = 0; k < 4; k++) v[k] = sh[k][0];
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
noalloc_partial(uint32_t n, const double *__restrict__ ux, const double *__restrict__ uy,
                const double *__restrict__ uz, const double *__restrict__ rho, double *__restrict__ partial) {
    __shared__ double sh[4][NOALLOC_THREADS];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = blockIdx.x * NOALLOC_THREADS + threadIdx.x; i < n; i += gridDim.x * NOALLOC_THREADS) {
        v[0] += ux[i];
        v[1] += uy[i];
        v[2] += uz[i];
        v[3] += rho[i];
    }
    sum4(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) partial[blockIdx.x * 4 + k] = v[k];
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
noalloc_final(int nblocks, uint32_t n, const double *__restrict__ partial, double *__restrict__ out) {
    __shared__ double sh[4][NOALLOC_THREADS];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += NOALLOC_THREADS)
        for (int k = 0; k < 4; k++) v[k] += partial[b * 4 + k];
    sum4(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) out[k] = v[k] / (double)n;
}

} // namespace

// the library's per-thread error text (rr_api.cu)
rr_status rr_internal_error(rr_status st, const char *fmt, ...);

extern "C" rr_status rr_diag_fields_noalloc(const double *rho, const double *ux, const double *uy,
                                            const double *uz, size_t n, double *out, void *stream) {
    if (!rho || !ux || !uy || !uz || !out)
        return rr_internal_error(RR_ERR_INVALID, "rr_diag_fields_noalloc: NULL field or output pointer");
    if (n == 0 || n > 2147483647u) // one 32-bit index per node
        return rr_internal_error(RR_ERR_INVALID,
                                 "rr_diag_fields_noalloc: n = %zu nodes; the preallocated reduction "
                                 "takes 1 to 2147483647 nodes",
                                 n);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return rr_internal_error(RR_ERR_CUDA, "rr_diag_fields_noalloc: no current CUDA device");
    }
    if (dev < 0 || dev >= MAX_DEVICES)
        return rr_internal_error(RR_ERR_UNSUPPORTED, "rr_diag_fields_noalloc: device %d >= %d", dev, MAX_DEVICES);
    double *scratch;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return rr_internal_error(RR_ERR_CUDA, "rr_diag_fields_noalloc: cudaGetSymbolAddress: %s",
                                         cudaGetErrorString(e));
            }
            g_scratch_addr[dev] = static_cast<double *>(p);
        }
        scratch = g_scratch_addr[dev];
    }
    const uint32_t nn = (uint32_t)n;
    int nb = (int)((nn + NOALLOC_THREADS - 1) / NOALLOC_THREADS);
    if (nb > NOALLOC_BLOCKS) nb = NOALLOC_BLOCKS;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    noalloc_partial<<<nb, NOALLOC_THREADS, 0, st>>>(nn, ux, uy, uz, rho, scratch);
    noalloc_final<<<1, NOALLOC_THREADS, 0, st>>>(nb, nn, scratch, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return rr_internal_error(RR_ERR_CUDA, "rr_diag_fields_noalloc: launch failed: %s", cudaGetErrorString(e));
    return RR_OK;
}
