// rr_pair.cuh -- two lattice nodes per thread in packed FP32 pairs.
//
// The node arithmetic of rr_node.cuh is written once over its compute type
// T.  F2 is a pair of FP32 values (two x-adjacent nodes) whose operations map
// to the packed FP32x2 instructions of sm_100-family GPUs (add/sub/mul/fma
// .rn.f32x2): one instruction does the work of two scalar FP32 instructions,
// which halves the issue slots the collision takes.  Each lane of an F2
// operation rounds exactly as the scalar FP32 operation does, and the
// compiler fuses the pair code's multiply-adds as it fuses the scalar code's
// (the same template code): a node computed in a pair gets the same bits as
// the same node computed alone (tests/pair_check.cu checks it on the GPU).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

namespace rr {

struct F2 {
    float2 v;
    F2() = default;
    __device__ __forceinline__ explicit F2(float2 a) : v(a) {}
    __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    // a constant in both lanes
    __device__ __forceinline__ explicit F2(double c) : v(make_float2((float)c, (float)c)) {}
    __device__ __forceinline__ explicit F2(float c) : v(make_float2(c, c)) {}
    __device__ __forceinline__ explicit F2(int c) : v(make_float2((float)c, (float)c)) {}
    __device__ __forceinline__ float lo() const { return v.x; }
    __device__ __forceinline__ float hi() const { return v.y; }
};

__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 operator-(F2 a) { return F2(make_float2(-a.v.x, -a.v.y)); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
    unsigned long long r;
    const unsigned long long x = *reinterpret_cast<const unsigned long long *>(&a.v);
    const unsigned long long y = *reinterpret_cast<const unsigned long long *>(&b.v);
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(x), "l"(y));
    return F2(*reinterpret_cast<const float2 *>(&r));
}
// IEEE division lane by lane (as the scalar FP32 division)
__device__ __forceinline__ F2 operator/(F2 a, F2 b) {
    return F2(make_float2(__fdiv_rn(a.v.x, b.v.x), __fdiv_rn(a.v.y, b.v.y)));
}
__device__ __forceinline__ F2 &operator+=(F2 &a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2 &operator-=(F2 &a, F2 b) { return a = a - b; }
__device__ __forceinline__ F2 &operator*=(F2 &a, F2 b) { return a = a * b; }
__device__ __forceinline__ F2 fma_(F2 a, F2 b, F2 c) { return F2(__ffma2_rn(a.v, b.v, c.v)); }

// two consecutive stored populations (the first at an even element offset)
// as an FP32 pair
template <typename S> __device__ __forceinline__ F2 ld_pair(const S *p);
template <> __device__ __forceinline__ F2 ld_pair(const float *p) {
    return F2(*reinterpret_cast<const float2 *>(p));
}
template <> __device__ __forceinline__ F2 ld_pair(const __half *p) {
    return F2(__half22float2(*reinterpret_cast<const __half2 *>(p)));
}
template <> __device__ __forceinline__ F2 ld_pair(const __nv_bfloat16 *p) {
    return F2(__bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(p)));
}

// Two consecutive stored elements (the first at an even element offset) as
// raw bits, the first element in the low half: 32 bits for FP16/BF16, 64 for
// FP32.  The aligned pair layout moves populations between lanes in this form.
template <typename S> struct PairWord { using W = uint32_t; };
template <> struct PairWord<float> { using W = unsigned long long; };

template <typename S> __device__ __forceinline__ typename PairWord<S>::W ld_word(const S *p) {
    return *reinterpret_cast<const typename PairWord<S>::W *>(p);
}
// one element into the low / the high half of a word
template <typename S> __device__ __forceinline__ typename PairWord<S>::W elem_lo(const S *p) {
    if constexpr (sizeof(S) == 2) return (uint32_t)*reinterpret_cast<const unsigned short *>(p);
    else return (unsigned long long)*reinterpret_cast<const uint32_t *>(p);
}
template <typename S> __device__ __forceinline__ typename PairWord<S>::W elem_hi(const S *p) {
    if constexpr (sizeof(S) == 2) return (uint32_t)*reinterpret_cast<const unsigned short *>(p) << 16;
    else return (unsigned long long)*reinterpret_cast<const uint32_t *>(p) << 32;
}
// (a's high element, b's low element): with a = (x-2, x-1), b = (x, x+1)
// the elements at x-1 and x
template <typename S>
__device__ __forceinline__ typename PairWord<S>::W join_word(typename PairWord<S>::W a, typename PairWord<S>::W b) {
    if constexpr (sizeof(S) == 2) return __byte_perm(a, b, 0x5432);
    else return (a >> 32) | (b << 32);
}
// the word's elements as FP32 (exact conversions, as ld_dev's)
template <typename S> __device__ __forceinline__ F2 word_f2(typename PairWord<S>::W w) {
    if constexpr (std::is_same<S, __half>::value) return F2(__half22float2(*reinterpret_cast<const __half2 *>(&w)));
    else if constexpr (std::is_same<S, __nv_bfloat16>::value)
        return F2(__bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&w)));
    else return F2(*reinterpret_cast<const float2 *>(&w));
}
// an FP32 pair as a word of the storage type, each element rounded to nearest
template <typename S> __device__ __forceinline__ typename PairWord<S>::W word_of(F2 v) {
    typename PairWord<S>::W w;
    if constexpr (std::is_same<S, __half>::value) *reinterpret_cast<__half2 *>(&w) = __float22half2_rn(v.v);
    else if constexpr (std::is_same<S, __nv_bfloat16>::value)
        *reinterpret_cast<__nv_bfloat162 *>(&w) = __float22bfloat162_rn(v.v);
    else *reinterpret_cast<float2 *>(&w) = v.v;
    return w;
}
// a word into two consecutive elements (the first at an even element
// offset): keep = 3 both (one aligned store), 1 the first only, 2 the second
// only
template <typename S> __device__ __forceinline__ void put_word(S *p, typename PairWord<S>::W w, uint32_t keep) {
    using W = typename PairWord<S>::W;
    using E = typename std::conditional<sizeof(S) == 2, unsigned short, uint32_t>::type;
    constexpr int SH = 8 * (int)sizeof(S);
    if (keep == 3u) *reinterpret_cast<W *>(p) = w;
    else if (keep == 1u) *reinterpret_cast<E *>(p) = (E)w;
    else *reinterpret_cast<E *>(p + 1) = (E)(w >> SH);
}

} // namespace rr
