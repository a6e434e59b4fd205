// rr_lattice.cuh -- compile-time D3Q19 / D3Q27 velocity sets and the
// Hermite coefficients of the recursive-regularized (RR) collision.
//
// Velocity orders follow the reference so that population exchange needs no
// permutation in the common case:
//   D3Q27: RR27V33_code_DNS_LES/initial.cu:67-69 (the CUDA channel code)
//   D3Q19: Taylor_Green/D3Q19RR.f90:75-77 (the only D3Q19 code)
// Weights: initial.cu:71-77 and D3Q19RR.f90:79-81.
//
// Everything here is constexpr; the kernels walk the populations with
// static_for so that every c_i, w_i and Hermite coefficient is an immediate
// and multiplications by 0 are never emitted.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

// the lattice and node arithmetic also compile as plain C++ (host checks)
#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline __attribute__((always_inline))
#endif

namespace rr {

template <typename F, int... I>
__host__ __device__ __forceinline__ void static_for_impl(F &&f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__host__ __device__ __forceinline__ void static_for(F &&f) {
    static_for_impl(f, std::make_integer_sequence<int, N>{});
}

struct D3Q27 {
    static constexpr int Q = 27;
    static constexpr int CX[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1,
                                   0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    static constexpr int CY[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0,
                                   -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    static constexpr int CZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1,
                                   1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    __host__ __device__ static constexpr double weight_of(int n) {
        return n == 0 ? 8.0 / 27.0 : n == 1 ? 2.0 / 27.0 : n == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
    }
};

struct D3Q19 {
    static constexpr int Q = 19;
    static constexpr int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0};
    static constexpr int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1};
    static constexpr int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    __host__ __device__ static constexpr double weight_of(int n) {
        return n == 0 ? 1.0 / 3.0 : n == 1 ? 1.0 / 18.0 : 1.0 / 36.0;
    }
};

template <typename L>
struct Lat {
    using Set = L; // host code indexes Set::CX etc. with run-time indices
    static constexpr int Q = L::Q;
    __host__ __device__ static constexpr int cx(int i) { return L::CX[i]; }
    __host__ __device__ static constexpr int cy(int i) { return L::CY[i]; }
    __host__ __device__ static constexpr int cz(int i) { return L::CZ[i]; }
    __host__ __device__ static constexpr int nnz(int i) {
        return (cx(i) != 0) + (cy(i) != 0) + (cz(i) != 0);
    }
    __host__ __device__ static constexpr double w(int i) { return L::weight_of(nnz(i)); }
    __host__ __device__ static constexpr int opp(int i) {
        for (int j = 0; j < Q; j++)
            if (cx(j) == -cx(i) && cy(j) == -cy(i) && cz(j) == -cz(i)) return j;
        return -1;
    }
    // "positive" member of each opposite pair: first non-zero component > 0
    __host__ __device__ static constexpr bool positive(int i) {
        return cx(i) > 0 || (cx(i) == 0 && (cy(i) > 0 || (cy(i) == 0 && cz(i) > 0)));
    }
    static constexpr int NPAIR = (Q - 1) / 2;
    __host__ __device__ static constexpr int pos(int k) {
        int n = 0;
        for (int i = 0; i < Q; i++)
            if (positive(i)) {
                if (n == k) return i;
                n++;
            }
        return -1;
    }
    __host__ __device__ static constexpr int rest() {
        for (int i = 0; i < Q; i++)
            if (nnz(i) == 0) return i;
        return -1;
    }

    // Second-order part: 1/2 sec_i(A) with
    //   sec = 2 (H110 A110 + H101 A101 + H011 A011) + H200 A200 + H020 A020 + H002 A002,
    //   H_ab = c_a c_b / cs^2 - delta_ab   (initial.cu:97-102, collision.cu:58-59).
    // Coefficient k of A in order (110, 101, 011, 200, 020, 002).
    __host__ __device__ static constexpr double hs(int i, int k) {
        return k == 0   ? 3.0 * cx(i) * cy(i)
               : k == 1 ? 3.0 * cx(i) * cz(i)
               : k == 2 ? 3.0 * cy(i) * cz(i)
               : k == 3 ? 0.5 * (3 * cx(i) * cx(i) - 1)
               : k == 4 ? 0.5 * (3 * cy(i) * cy(i) - 1)
                        : 0.5 * (3 * cz(i) * cz(i) - 1);
    }

    // Third-order part: 1/2 thir_i(B) = sum_k ht(i,k) * b_k with b_k = (sqrt3/2) B_k
    // for k in (210, 201, 021, 120, 012, 102) and the H111 term as ht(i,6) * t111,
    // t111 = 3 sqrt3 B111 (collision.cu:60-61, initial.cu:104-110).  H210/sqrt3 =
    // c_y (3 c_x^2 - 1), and so on.  D3Q19 keeps only the admissible combinations
    // H210 +- H012, H102 +- H120, H021 +- H201 with the (-) terms weighted 1/3
    // (Taylor_Green/D3Q19RR.f90:131-136, 373-378), which gives the integer
    // coefficients (4 A + 2 C)/3 below and no H111 term.
    __host__ __device__ static constexpr int h3(int i, int k) { // H_k / sqrt3
        return k == 0   ? cy(i) * (3 * cx(i) * cx(i) - 1)
               : k == 1 ? cz(i) * (3 * cx(i) * cx(i) - 1)
               : k == 2 ? cz(i) * (3 * cy(i) * cy(i) - 1)
               : k == 3 ? cx(i) * (3 * cy(i) * cy(i) - 1)
               : k == 4 ? cy(i) * (3 * cz(i) * cz(i) - 1)
               : k == 5 ? cx(i) * (3 * cz(i) * cz(i) - 1)
                        : cx(i) * cy(i) * cz(i);
    }
    __host__ __device__ static constexpr double ht(int i, int k) {
        if (Q == 27) return (double)h3(i, k);
        // D3Q19: pairs (210, 012), (102, 120), (021, 201)
        int partner = k == 0 ? 4 : k == 4 ? 0 : k == 5 ? 3 : k == 3 ? 5 : k == 2 ? 1 : k == 1 ? 2 : 6;
        if (partner == 6) return 0.0;
        return (4.0 * h3(i, k) + 2.0 * h3(i, partner)) / 3.0;
    }
};

using L27 = Lat<D3Q27>;
using L19 = Lat<D3Q19>;

// permutation between the Fortran D3Q27 order (Taylor_Green/D3Q27RR.f90:69-71,
// Cavity/para.f90:126-128) and the CUDA order used internally:
// fortran_to_cuda[j] = internal index of Fortran population j
constexpr int FORTRAN_TO_CUDA_27[27] = {0,  1,  3,  2,  4,  5,  6,  7,  10, 8,  9,  11, 15, 13,
                                        17, 12, 16, 14, 18, 19, 23, 22, 26, 20, 24, 21, 25};

} // namespace rr
