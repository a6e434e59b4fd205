/* Host stand-in for the CUDA runtime header, so that the reference's kernel
 * sources (RR27V33_code_DNS_LES/{globals,collision,streaming,macrovar,BC,LES}.cu)
 * and its output routines (output.cu) compile as plain C++ for the CPU
 * oracle.  TEST INFRASTRUCTURE ONLY.
 * Kernels become ordinary functions; the thread/block coordinates are
 * thread-local variables that ref_driver.cpp sets before each call. */
#ifndef RR_REF_SHIM_CUDA_RUNTIME_H
#define RR_REF_SHIM_CUDA_RUNTIME_H
#include <stdio.h>
#include <stdlib.h>

#define __global__
#define __device__
#define __constant__
#define __host__

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

typedef int cudaError_t;
static inline const char *cudaGetErrorString(cudaError_t) { return "host shim"; }

/* the output routines (output.cu) copy the fields "device to host": on the
 * host a plain copy */
#include <string.h>
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3 };
static const cudaError_t cudaSuccess = 0;
static inline cudaError_t cudaMemcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind) {
    memcpy(dst, src, bytes);
    return cudaSuccess;
}
#endif
