// rr_node.cuh -- per-node arithmetic of the recursive-regularized (RR)
// collision, the regularized wall closure and the moments.
//
// Populations are carried as deviations d_i = f_i / w_i - 1 (the "shifted"
// form): every sum below is a sum of small numbers, which keeps FP32 compute
// and FP16/BF16 storage accurate, and the arithmetic is the same for FP64.
//
// The reference evaluates, per node (collision.cu:41-119, BC.cu:30-125):
//   feq_i   = w_i rho (1 + H1.u^ + 1/2 (sec_i(a2) + thir_i(a3)))
//   Fbar_i  = 1/2 (c_i - u).F / cs^2
//   a2neq   = sum_i H2_i (f_i + Fbar_i feq_i) - rho u^ u^
//   a3neq   = recursive from a2neq and u^ (collision.cu:88-94)
//   fneq_i  = w_i 1/2 (sec_i(a2neq) + thir_i(a3neq))
//   collide : f_i <- feq_i + (1 - 1/tau) fneq_i + Fbar_i feq_i
//   wall    : f_i <- feq_i + fneq_i - Fbar_i feq_i   (entering i only)
// Here the same quantities are formed once per opposite pair (i, ibar):
// H2 terms are even, H1/H3 terms odd, so each pair needs one even and one odd
// polynomial.  Without a body force the equilibrium and non-equilibrium
// Hermite coefficients are merged before the per-pair evaluation.
#pragma once

#include <cmath>

#include "rr_lattice.cuh"

namespace rr {

// a * b + c with one rounding, for every compute type of the node arithmetic
// (the packed FP32 pair of rr_pair.cuh has its own overload): the products
// that should fuse say so, rather than leaving it to contraction.
__host__ __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
__host__ __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }

template <typename T>
struct Mom {
    T drho;               // sum f - 1
    T jx, jy, jz;         // sum c f
    T pxx, pyy, pzz;      // sum w c_a c_a d
    T pxy, pxz, pyz;      // sum w c_a c_b d
};

// zeroth, first and second moments from the deviations (macrovar.cu:4-31
// for rho and j; the second moments feed a2neq, collision.cu:73-78)
template <class LT, typename T>
__host__ __device__ __forceinline__ Mom<T> moments_generic(const T (&d)[LT::Q]) {
    Mom<T> m;
    constexpr int r = LT::rest();
    m.drho = T(LT::w(r)) * d[r];
    m.jx = m.jy = m.jz = T(0);
    m.pxx = m.pyy = m.pzz = m.pxy = m.pxz = m.pyz = T(0);
    static_for<LT::NPAIR>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int i = LT::pos(k);
        constexpr int o = LT::opp(i);
        constexpr int cx = LT::cx(i), cy = LT::cy(i), cz = LT::cz(i);
        const T w = T(LT::w(i));
        T ws = w * (d[i] + d[o]);
        T wd = w * (d[i] - d[o]);
        m.drho += ws;
        if constexpr (cx > 0) m.jx += wd;
        if constexpr (cx < 0) m.jx -= wd;
        if constexpr (cy > 0) m.jy += wd;
        if constexpr (cy < 0) m.jy -= wd;
        if constexpr (cz > 0) m.jz += wd;
        if constexpr (cz < 0) m.jz -= wd;
        if constexpr (cx != 0) m.pxx += ws;
        if constexpr (cy != 0) m.pyy += ws;
        if constexpr (cz != 0) m.pzz += ws;
        if constexpr (cx * cy > 0) m.pxy += ws;
        if constexpr (cx * cy < 0) m.pxy -= ws;
        if constexpr (cx * cz > 0) m.pxz += ws;
        if constexpr (cx * cz < 0) m.pxz -= ws;
        if constexpr (cy * cz > 0) m.pyz += ws;
        if constexpr (cy * cz < 0) m.pyz -= ws;
    });
    return m;
}

// sum_k hs(i,k) A_k : 1/2 sec_i(A)
template <class LT, int I, typename T>
__host__ __device__ __forceinline__ T even_poly(const T (&A)[6]) {
    T s = T(0);
    bool first = true;
    static_for<6>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr double h = LT::hs(I, k);
        if constexpr (h != 0.0) {
            if constexpr (h == 1.0) {
                s = first ? A[k] : s + A[k];
            } else if constexpr (h == -1.0) {
                s = first ? -A[k] : s - A[k];
            } else {
                s = first ? T(h) * A[k] : fma_(T(h), A[k], s);
            }
            first = false;
        }
    });
    return s;
}

// 1/2 thir_i(B), plus 3 rho c.u from B[7..9] when LINEAR
template <class LT, int I, typename T, bool LINEAR = true>
__host__ __device__ __forceinline__ T odd_poly(const T (&B)[10]) {
    // B[0..5] = b210 b201 b021 b120 b012 b102, B[6] = t111, B[7..9] = 3 rho u
    T s = T(0);
    bool first = true;
    auto add = [&](double h, T v) {
        if (h == 0.0) return;
        if (h == 1.0) s = first ? v : s + v;
        else if (h == -1.0) s = first ? -v : s - v;
        else s = first ? T(h) * v : fma_(T(h), v, s);
        first = false;
    };
    if constexpr (LINEAR) {
        add((double)LT::cx(I), B[7]);
        add((double)LT::cy(I), B[8]);
        add((double)LT::cz(I), B[9]);
    }
    static_for<7>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr double h = LT::ht(I, k);
        if constexpr (h != 0.0) add(h, B[k]);
    });
    return s;
}

// second-order moments of the non-equilibrium part, without the force
// correction: sum_i H2_i f_i - rho u^ u^  (collision.cu:73-86) in the order
// (110, 101, 011, 200, 020, 002)
template <typename T>
__host__ __device__ __forceinline__ void aneq_base(const Mom<T> &m, T rho, T ux, T uy, T uz, T (&n)[6]) {
    const T r3 = T(3) * rho;
    const T rx = -(r3 * ux), ry = -(r3 * uy), rz = -(r3 * uz);
    n[0] = fma_(rx, uy, T(3) * m.pxy);
    n[1] = fma_(rx, uz, T(3) * m.pxz);
    n[2] = fma_(ry, uz, T(3) * m.pyz);
    n[3] = fma_(rx, ux, fma_(T(3), m.pxx, -m.drho));
    n[4] = fma_(ry, uy, fma_(T(3), m.pyy, -m.drho));
    n[5] = fma_(rz, uz, fma_(T(3), m.pzz, -m.drho));
}

// third-order coefficients (recursive a3neq, collision.cu:88-94) scaled for
// odd_poly: b_k = (sqrt3/2) * scale * a3_k, t111 = 3 sqrt3 * scale * a111
template <typename T>
__host__ __device__ __forceinline__ void third_from_second(const T (&n)[6], T ux, T uy, T uz, T scale,
                                                  T (&B)[10]) {
    const T s15 = T(1.5) * scale;
    const T x2 = T(2) * ux, y2 = T(2) * uy, z2 = T(2) * uz;
    B[0] = s15 * fma_(n[3], uy, x2 * n[0]); // 210
    B[1] = s15 * fma_(n[3], uz, x2 * n[1]); // 201
    B[2] = s15 * fma_(n[4], uz, y2 * n[2]); // 021
    B[3] = s15 * fma_(n[4], ux, y2 * n[0]); // 120
    B[4] = s15 * fma_(n[5], uy, z2 * n[2]); // 012
    B[5] = s15 * fma_(n[5], ux, z2 * n[1]); // 102
    B[6] = (T(9) * scale) * fma_(n[0], uz, fma_(n[1], uy, n[2] * ux));
}

// equilibrium Hermite coefficients: A = rho u^ u^ (3 rho u_a u_b), b = (sqrt3/2)
// rho u^ u^ u^ (4.5 rho u_a^2 u_b), t111 = 3 sqrt3 rho u^ v^ w^ (27 rho u v w)
template <typename T>
__host__ __device__ __forceinline__ void eq_coeffs(T rho, T ux, T uy, T uz, T (&A)[6], T (&B)[10]) {
    const T r3 = T(3) * rho, r45 = T(4.5) * rho;
    const T rx = r3 * ux, ry = r3 * uy, rz = r3 * uz;
    const T qx = r45 * ux * ux, qy = r45 * uy * uy, qz = r45 * uz * uz;
    A[0] = rx * uy;
    A[1] = rx * uz;
    A[2] = ry * uz;
    A[3] = rx * ux;
    A[4] = ry * uy;
    A[5] = rz * uz;
    B[0] = qx * uy;
    B[1] = qx * uz;
    B[2] = qy * uz;
    B[3] = qy * ux;
    B[4] = qz * uy;
    B[5] = qz * ux;
    B[6] = T(9) * A[0] * uz;
    B[7] = rx;
    B[8] = ry;
    B[9] = rz;
}

// Force correction sum_i H2_ab,i Fbar_i feq_i (the f + Fbar feq term of
// collision.cu:73-78), from the equilibrium coefficients.
template <class LT, typename T>
__host__ __device__ __forceinline__ void force_correction(T drho_eq, const T (&Aq)[6], const T (&Bq)[10],
                                                 T Fe, T Fx, T Fy, T Fz, T (&C)[6]) {
    constexpr int r = LT::rest();
    T Ee0 = drho_eq + even_poly<LT, r>(Aq);
    T ef0 = T(LT::w(r)) * (T(1) + Ee0) * Fe;
    static_for<6>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr double h = LT::hs(r, k) * (k < 3 ? 1.0 : 2.0);
        if constexpr (h != 0.0) C[k] = T(h) * ef0;
        else C[k] = T(0);
    });
    static_for<LT::NPAIR>([&](auto pc) {
        constexpr int p = decltype(pc)::value;
        constexpr int i = LT::pos(p);
        T Ee = drho_eq + even_poly<LT, i>(Aq);
        T Eo = odd_poly<LT, i>(Bq);
        T Fo = T(1.5) * (T(LT::cx(i)) * Fx + T(LT::cy(i)) * Fy + T(LT::cz(i)) * Fz);
        // sum over the pair of w E Fbar = 2 w ((1 + Ee) Fe + Eo Fo)
        T ef = T(2.0 * LT::w(i)) * ((T(1) + Ee) * Fe + Eo * Fo);
        static_for<6>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            // hs carries 3 c_a c_b for k < 3 (H110 = 3 c_a c_b) and
            // 1/2 (3 c_a^2 - 1) for k >= 3 (H200 = 3 c_a^2 - 1)
            constexpr double h = LT::hs(i, k) * (k < 3 ? 1.0 : 2.0);
            if constexpr (h != 0.0) C[k] += T(h) * ef;
        });
    });
}

// RR collision of one node.  d: post-stream deviations (in), post-collision
// deviations (out).  m: moments of d.  (drho_eq, u): the macroscopic state the
// equilibrium is built from (normally drho_eq = m.drho and u = (j + F/2)/rho;
// the first collision after a state upload takes them from the caller, as the
// reference's first step takes init_arrays' macros, initial.cu:278-313).
template <class LT, typename T, bool FORCE>
__host__ __device__ __forceinline__ void collide_generic(T (&d)[LT::Q], const Mom<T> &m, T drho_eq, T ux, T uy,
                                                         T uz, T om1, T Fx, T Fy, T Fz) {
    const T rho = T(1) + drho_eq;
    T n[6];
    aneq_base(m, rho, ux, uy, uz, n);
    T Aq[6], Bq[10];
    eq_coeffs(rho, ux, uy, uz, Aq, Bq);
    T Fe = T(0);
    if constexpr (FORCE) {
        Fe = T(-1.5) * (ux * Fx + uy * Fy + uz * Fz);
        T C[6];
        force_correction<LT>(drho_eq, Aq, Bq, Fe, Fx, Fy, Fz, C);
#pragma unroll
        for (int k = 0; k < 6; k++) n[k] += C[k];
    }
    if constexpr (!FORCE) {
        // merged coefficients: rho a2 + (1 - 1/tau) a2neq, same for third order
        T A[6], B[10];
#pragma unroll
        for (int k = 0; k < 6; k++) A[k] = fma_(om1, n[k], Aq[k]);
        T Bn[10];
        third_from_second(n, ux, uy, uz, om1, Bn);
#pragma unroll
        for (int k = 0; k < 7; k++) B[k] = Bq[k] + Bn[k];
        B[7] = Bq[7];
        B[8] = Bq[8];
        B[9] = Bq[9];
        constexpr int r = LT::rest();
        d[r] = drho_eq + even_poly<LT, r>(A);
        static_for<LT::NPAIR>([&](auto pc) {
            constexpr int p = decltype(pc)::value;
            constexpr int i = LT::pos(p);
            constexpr int o = LT::opp(i);
            T e = drho_eq + even_poly<LT, i>(A);
            T od = odd_poly<LT, i>(B);
            d[i] = e + od;
            d[o] = e - od;
        });
    } else {
        T An[6], Bn[10];
#pragma unroll
        for (int k = 0; k < 6; k++) An[k] = om1 * n[k];
        third_from_second(n, ux, uy, uz, om1, Bn);
        constexpr int r = LT::rest();
        {
            T Ee = drho_eq + even_poly<LT, r>(Aq);
            d[r] = Ee + (T(1) + Ee) * Fe + even_poly<LT, r>(An);
        }
        static_for<LT::NPAIR>([&](auto pc) {
            constexpr int p = decltype(pc)::value;
            constexpr int i = LT::pos(p);
            constexpr int o = LT::opp(i);
            T Ee = drho_eq + even_poly<LT, i>(Aq);
            T Eo = odd_poly<LT, i>(Bq);
            T Fo = T(1.5) * (T(LT::cx(i)) * Fx + T(LT::cy(i)) * Fy + T(LT::cz(i)) * Fz);
            T efe = (T(1) + Ee) * Fe + Eo * Fo;
            T efo = (T(1) + Ee) * Fo + Eo * Fe;
            T ne = even_poly<LT, i>(An);
            T no = odd_poly<LT, i, T, false>(Bn);
            T e = Ee + efe + ne;
            T od = Eo + efo + no;
            d[i] = e + od;
            d[o] = e - od;
        });
    }
}

} // namespace rr

#include "rr_node27.cuh"

namespace rr {

// D3Q27 goes through the hand-factored forms of rr_node27.cuh (same
// arithmetic, shared partial sums); D3Q19 and the forced collision through
// the generic pair loop above
template <class LT, typename T>
__host__ __device__ __forceinline__ Mom<T> moments(const T (&d)[LT::Q]) {
    if constexpr (LT::Q == 27) return moments27(d);
    else return moments_generic<LT>(d);
}

template <class LT, typename T, bool FORCE>
__host__ __device__ __forceinline__ void collide(T (&d)[LT::Q], const Mom<T> &m, T drho_eq, T ux, T uy,
                                                 T uz, T om1, T Fx, T Fy, T Fz) {
    if constexpr (LT::Q == 27 && !FORCE) collide27(d, m, drho_eq, ux, uy, uz, om1);
    else if constexpr (LT::Q == 27) collide27_forced(d, m, drho_eq, ux, uy, uz, om1, Fx, Fy, Fz);
    else collide_generic<LT, T, FORCE>(d, m, drho_eq, ux, uy, uz, om1, Fx, Fy, Fz);
}

// velocity from the moments with the half-force shift (macrovar.cu:25-28)
template <typename T>
__host__ __device__ __forceinline__ void velocity(const Mom<T> &m, T Fx, T Fy, T Fz, T &ux, T &uy, T &uz) {
    const T inv = T(1) / (T(1) + m.drho);
    ux = fma_(T(0.5), Fx, m.jx) * inv;
    uy = fma_(T(0.5), Fy, m.jy) * inv;
    uz = fma_(T(0.5), Fz, m.jz) * inv;
}

// Regularized wall closure of one node (RRBC, BC.cu:4-126; Cavity
// streaming.f90:100-140): moments of the current populations, then the
// populations flagged in `mask` are rebuilt as feq + fneq - Fbar feq.
// CMASK is a compile-time superset of `mask` (the entering set of a face
// known at compile time): populations outside it generate no code.
template <class LT, typename T, bool FORCE, uint32_t CMASK = 0xFFFFFFFFu>
__host__ __device__ __forceinline__ void regularize(T (&d)[LT::Q], uint32_t mask, T Fx, T Fy, T Fz) {
    Mom<T> m = moments<LT>(d);
    T ux, uy, uz;
    velocity(m, Fx, Fy, Fz, ux, uy, uz);
    const T rho = T(1) + m.drho;
    T n[6];
    aneq_base(m, rho, ux, uy, uz, n);
    T Aq[6], Bq[10];
    eq_coeffs(rho, ux, uy, uz, Aq, Bq);
    T Fe = T(0);
    if constexpr (FORCE) {
        Fe = T(-1.5) * (ux * Fx + uy * Fy + uz * Fz);
        T C[6];
        force_correction<LT>(m.drho, Aq, Bq, Fe, Fx, Fy, Fz, C);
#pragma unroll
        for (int k = 0; k < 6; k++) n[k] += C[k];
    }
    T Bn[10];
    third_from_second(n, ux, uy, uz, T(1), Bn);
    static_for<LT::Q>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        if constexpr (((CMASK >> i) & 1u) != 0)
        if ((mask >> i) & 1u) {
            T Ee = m.drho + even_poly<LT, i>(Aq);
            T Eo = odd_poly<LT, i>(Bq);
            T v = Ee + Eo + even_poly<LT, i>(n) + odd_poly<LT, i, T, false>(Bn);
            if constexpr (FORCE) {
                T Fo = T(1.5) * (T(LT::cx(i)) * Fx + T(LT::cy(i)) * Fy + T(LT::cz(i)) * Fz);
                v -= (T(1) + Ee + Eo) * (Fe + Fo);
            }
            d[i] = v;
        }
    });
}

} // namespace rr
