// rr_aux.h -- launchers of the FP64 statistics kernels (rr_aux.cu)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "rr_dispatch.h"

namespace rr {

// upper bound of the partial-sum blocks of the domain means
constexpr int DIAG_MAX_BLOCKS = 1024;
int diag_blocks(uint32_t n);

// diag_flow's {umean, vmean, wmean, rhomean} (output.cu:24-35); `partial`
// holds 4 * diag_blocks(n) doubles of scratch
cudaError_t launch_diag(uint32_t n, const double *ux, const double *uy, const double *uz,
                        const double *rho, double *partial, double *out, cudaStream_t st);

// output_profile's per-plane statistics, 12 * ny doubles (see rr_api.h)
cudaError_t launch_profile(const Geom &g, double ystar, const double *ux, const double *uy,
                           const double *uz, const double *taut, double *out, cudaStream_t st);

cudaError_t launch_accumulate(int m, const double *prof, double *acc, cudaStream_t st);

// the trip force of one step (or the uniform force when trip == 0) into ff
// (3 arrays of stride); amp = (100 beta / LY) sin(2 pi n / 2000)
cudaError_t launch_trip_force(double *ff, unsigned long long stride, int LX, int LY, int LZ, int trip, double amp,
                              double phase, const double F[3], cudaStream_t st);

// the y = 0 and y = ny-1 rows of a field (N doubles) into out[side][z][x]
cudaError_t launch_wall_rows(const Geom &g, const double *field, double *out, cudaStream_t st);

} // namespace rr
