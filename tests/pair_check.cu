// pair_check.cu -- the packed FP32-pair node arithmetic (csrc/rr_pair.cuh)
// against the scalar FP32 node arithmetic on the GPU, bit for bit: moments,
// velocity, the second- and third-order coefficients, the full collision
// (force-free and forced, D3Q27) and the 16-bit stores of a pair as aligned
// words (stochastic and nearest rounding), for 65,536 random node pairs.  Built with
// the library's flags and run by tests/test_gpu_pair.py; prints the mismatch
// bits (0: none) and exits 1 on a mismatch.
#include <cstdio>
#include <cstdint>
#include "rr_kernels.cuh"
using namespace rr;

__device__ float rnd(uint32_t s) { return (float)(mix32(s) & 0xFFFFFF) / 16777216.0f - 0.5f; }

template <bool FORCE>
__global__ void check(int *bad, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float da[27], db[27];
    F2 d2[27];
    for (int i = 0; i < 27; i++) {
        da[i] = 0.02f * rnd(t * 64 + i);
        db[i] = 0.02f * rnd(t * 64 + 32 + i);
        d2[i] = F2(da[i], db[i]);
    }
    const float Fx = 1e-5f, Fy = -2e-6f, Fz = 3e-6f;
    Mom<float> ma = moments<L27>(da), mb = moments<L27>(db);
    Mom<F2> m2 = moments<L27>(d2);
    const float *pa = &ma.drho, *pb = &mb.drho;
    const F2 *p2 = &m2.drho;
    for (int k = 0; k < 10; k++)
        if (__float_as_uint(pa[k]) != __float_as_uint(p2[k].lo()) || __float_as_uint(pb[k]) != __float_as_uint(p2[k].hi()))
            atomicOr(bad, 1);
    float uxa, uya, uza, uxb, uyb, uzb;
    F2 ux2, uy2, uz2;
    velocity(ma, Fx, Fy, Fz, uxa, uya, uza);
    velocity(mb, Fx, Fy, Fz, uxb, uyb, uzb);
    velocity(m2, F2(Fx), F2(Fy), F2(Fz), ux2, uy2, uz2);
    if (__float_as_uint(uxa) != __float_as_uint(ux2.lo()) || __float_as_uint(uzb) != __float_as_uint(uz2.hi())) atomicOr(bad, 2);
    const float om1 = 1.0f - 1.0f / 0.55f;
    collide<L27, float, FORCE>(da, ma, ma.drho, uxa, uya, uza, om1, Fx, Fy, Fz);
    collide<L27, float, FORCE>(db, mb, mb.drho, uxb, uyb, uzb, om1, Fx, Fy, Fz);
    collide<L27, F2, FORCE>(d2, m2, m2.drho, ux2, uy2, uz2, F2(om1), F2(Fx), F2(Fy), F2(Fz));
    for (int i = 0; i < 27; i++)
        if (__float_as_uint(da[i]) != __float_as_uint(d2[i].lo()) || __float_as_uint(db[i]) != __float_as_uint(d2[i].hi()))
            atomicOr(bad, 4);
    // the pieces of the collision
    float nn[6]; F2 n2[6];
    aneq_base(ma, 1.0f + ma.drho, uxa, uya, uza, nn);
    aneq_base(m2, F2(1.0f) + m2.drho, ux2, uy2, uz2, n2);
    for (int k = 0; k < 6; k++) if (__float_as_uint(nn[k]) != __float_as_uint(n2[k].lo())) atomicOr(bad, 8);
    float Aq[6], Bq[10]; F2 Aq2[6], Bq2[10];
    eq_coeffs(1.0f + ma.drho, uxa, uya, uza, Aq, Bq);
    eq_coeffs(F2(1.0f) + m2.drho, ux2, uy2, uz2, Aq2, Bq2);
    for (int k = 0; k < 6; k++) if (__float_as_uint(Aq[k]) != __float_as_uint(Aq2[k].lo())) atomicOr(bad, 16);
    for (int k = 0; k < 10; k++) if (__float_as_uint(Bq[k]) != __float_as_uint(Bq2[k].lo())) atomicOr(bad, 32);
    float Bn[10]; F2 Bn2[10];
    third_from_second(nn, uxa, uya, uza, om1, Bn);
    third_from_second(n2, ux2, uy2, uz2, F2(om1), Bn2);
    for (int k = 0; k < 7; k++) if (__float_as_uint(Bn[k]) != __float_as_uint(Bn2[k].lo())) atomicOr(bad, 64);
}

// the FP16 / BF16 stores with stochastic rounding: a node pair through
// store_pair against each node through store_sr_pairs (its own rounding stream)
template <typename S>
__global__ void check_store(int *bad, int n, S *a, S *b) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const unsigned long long stride = 2ull * n;
    const uint32_t idx = 2u * t; // the pair's first node (even, aligned), as in the steps
    float da[27], db[27];
    F2 d2[27];
    for (int i = 0; i < 27; i++) {
        da[i] = 0.02f * rnd(t * 64 + i);
        db[i] = 0.02f * rnd(t * 64 + 32 + i);
        d2[i] = F2(da[i], db[i]);
    }
    const uint32_t sa = mix32(idx * 7u + 1u), sb = mix32(idx * 7u + 8u);
    store_sr_pairs<L27, S, float>(da, sa, [&](int i) { return a + i * stride + idx; });
    store_sr_pairs<L27, S, float>(db, sb, [&](int i) { return a + i * stride + idx + 1; });
    S *dst[27];
    for (int i = 0; i < 27; i++) dst[i] = b + i * stride;
    store_pair<L27, S>(dst, idx, d2, true, sa, sb);
    for (int i = 0; i < 27; i++)
        for (int k = 0; k < 2; k++) {
            const unsigned short x = *reinterpret_cast<unsigned short *>(a + i * stride + idx + k);
            const unsigned short y = *reinterpret_cast<unsigned short *>(b + i * stride + idx + k);
            if (x != y) atomicOr(bad, 128);
        }
    // nearest rounding: one word per population against two element stores
    S *dn[27];
    for (int i = 0; i < 27; i++) dn[i] = b + i * stride;
    store_pair<L27, S>(dn, idx, d2, false, 0u, 0u);
    for (int i = 0; i < 27; i++) {
        const S ea = (S)da[i], eb = (S)db[i];
        const unsigned short x0 = *reinterpret_cast<const unsigned short *>(&ea);
        const unsigned short x1 = *reinterpret_cast<const unsigned short *>(&eb);
        const unsigned short y0 = *reinterpret_cast<unsigned short *>(b + i * stride + idx);
        const unsigned short y1 = *reinterpret_cast<unsigned short *>(b + i * stride + idx + 1);
        if (x0 != y0 || x1 != y1) atomicOr(bad, 256);
    }
    // one node of the pair only (keep 1: the first, 2: the second): the other
    // element keeps what was there
    for (int keep = 1; keep <= 2; keep++) {
        for (int i = 0; i < 27; i++) {
            *reinterpret_cast<unsigned short *>(b + i * stride + idx) = 0x7777u;
            *reinterpret_cast<unsigned short *>(b + i * stride + idx + 1) = 0x7777u;
        }
        store_pair<L27, S, true>(dn, idx, d2, false, 0u, 0u, (uint32_t)keep);
        for (int i = 0; i < 27; i++) {
            const S ea = (S)da[i], eb = (S)db[i];
            const unsigned short w0 = keep == 1 ? *reinterpret_cast<const unsigned short *>(&ea) : 0x7777u;
            const unsigned short w1 = keep == 2 ? *reinterpret_cast<const unsigned short *>(&eb) : 0x7777u;
            if (*reinterpret_cast<unsigned short *>(b + i * stride + idx) != w0 ||
                *reinterpret_cast<unsigned short *>(b + i * stride + idx + 1) != w1)
                atomicOr(bad, 512);
        }
    }
}

int main() {
    int *d, h[2] = {-1, -1};
    if (cudaMalloc(&d, 8) != cudaSuccess || cudaMemset(d, 0, 8) != cudaSuccess) return 2;
    const int n = 1 << 16;
    check<false><<<n / 256, 256>>>(d, n);
    check<true><<<n / 256, 256>>>(d + 1, n);
    // 27 populations x 2 n nodes, twice, per 16-bit type
    const size_t elems = 27ull * 2ull * n;
    __half *ha, *hb;
    __nv_bfloat16 *ba, *bb;
    if (cudaMalloc(&ha, 2 * elems * sizeof(__half)) != cudaSuccess) return 2;
    if (cudaMalloc(&ba, 2 * elems * sizeof(__nv_bfloat16)) != cudaSuccess) return 2;
    hb = ha + elems;
    bb = ba + elems;
    check_store<__half><<<n / 256, 256>>>(d, n, ha, hb);
    check_store<__nv_bfloat16><<<n / 256, 256>>>(d + 1, n, ba, bb);
    if (cudaMemcpy(h, d, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    cudaFree(d);
    cudaFree(ha);
    cudaFree(ba);
    printf("pair vs scalar mismatch bits: force-free / FP16 stores %d, forced / BF16 stores %d "
           "(1 moments, 2 velocity, 4 collision, 8 aneq, 16 Aq, 32 Bq, 64 Bn, 128 stochastic stores, "
           "256 nearest stores, 512 one node of a pair)\n", h[0], h[1]);
    return (h[0] || h[1]) ? 1 : 0;
}
