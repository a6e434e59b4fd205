// rr_node27.cuh -- D3Q27 (internal order = RR27V33_code_DNS_LES/initial.cu:67-69)
// moments and force-free RR collision with shared partial sums.
//
// Same quantities as moments_generic / collide_generic of rr_node.cuh; the
// populations are grouped by class (3 axis pairs, 2 edge pairs per
// coordinate plane, 4 corner pairs) so that the sums common to a class are
// formed once.  Floating-point sums are not reassociated by the compiler,
// so this factoring has to be written out.
//
// Population pairs (positive member / opposite):
//   axis   1/3 (x)  2/4 (y)  5/6 (z)
//   xy     7 (1,1,0)/9    10 (1,-1,0)/8
//   xz     11 (1,0,1)/17  15 (1,0,-1)/13
//   yz     12 (0,1,1)/18  16 (0,1,-1)/14
//   corner 19 (1,1,1)/25  23 (1,1,-1)/21  22 (1,-1,1)/24  26 (1,-1,-1)/20
#pragma once

namespace rr {

template <typename T>
__host__ __device__ __forceinline__ Mom<T> moments27(const T (&d)[27]) {
    const T w0 = T(8.0 / 27.0), w1 = T(2.0 / 27.0), w2 = T(1.0 / 54.0), w3 = T(1.0 / 216.0);
    // axis pairs: sums s, differences g
    const T sx = d[1] + d[3], gx = d[1] - d[3];
    const T sy = d[2] + d[4], gy = d[2] - d[4];
    const T sz = d[5] + d[6], gz = d[5] - d[6];
    // edge pairs, combined per plane
    const T s7 = d[7] + d[9], g7 = d[7] - d[9], s10 = d[10] + d[8], g10 = d[10] - d[8];
    const T s11 = d[11] + d[17], g11 = d[11] - d[17], s15 = d[15] + d[13], g15 = d[15] - d[13];
    const T s12 = d[12] + d[18], g12 = d[12] - d[18], s16 = d[16] + d[14], g16 = d[16] - d[14];
    const T Sxy = s7 + s10, Dxy = s7 - s10, Jx_xy = g7 + g10, Jy_xy = g7 - g10;
    const T Sxz = s11 + s15, Dxz = s11 - s15, Jx_xz = g11 + g15, Jz_xz = g11 - g15;
    const T Syz = s12 + s16, Dyz = s12 - s16, Jy_yz = g12 + g16, Jz_yz = g12 - g16;
    // corner pairs
    const T s19 = d[19] + d[25], g19 = d[19] - d[25];
    const T s23 = d[23] + d[21], g23 = d[23] - d[21];
    const T s22 = d[22] + d[24], g22 = d[22] - d[24];
    const T s26 = d[26] + d[20], g26 = d[26] - d[20];
    const T ca = s19 + s23, cb = s22 + s26, cc = s19 - s23, ce = s22 - s26;
    const T ga = g19 + g23, gb = g22 + g26, gc = g19 - g23, ge = g22 - g26;
    const T Sc = ca + cb;                    // every corner
    const T Pxy_c = ca - cb, Pxz_c = cc + ce, Pyz_c = cc - ce;
    const T Jx_c = ga + gb, Jy_c = ga - gb, Jz_c = gc + ge;
    Mom<T> m;
    const T Se = Sxy + Sxz + Syz;
    const T c3 = w3 * Sc;
    m.drho = fma_(w0, d[0], fma_(w1, sx + sy + sz, fma_(w2, Se, c3)));
    m.jx = fma_(w1, gx, fma_(w2, Jx_xy + Jx_xz, w3 * Jx_c));
    m.jy = fma_(w1, gy, fma_(w2, Jy_xy + Jy_yz, w3 * Jy_c));
    m.jz = fma_(w1, gz, fma_(w2, Jz_xz + Jz_yz, w3 * Jz_c));
    m.pxx = fma_(w1, sx, fma_(w2, Sxy + Sxz, c3));
    m.pyy = fma_(w1, sy, fma_(w2, Sxy + Syz, c3));
    m.pzz = fma_(w1, sz, fma_(w2, Sxz + Syz, c3));
    m.pxy = fma_(w2, Dxy, w3 * Pxy_c);
    m.pxz = fma_(w2, Dxz, w3 * Pxz_c);
    m.pyz = fma_(w2, Dyz, w3 * Pyz_c);
    return m;
}

// Every population of a D3Q27 node from Hermite coefficients: with K the
// density deviation, A (110, 101, 011, 200, 020, 002) the second-order and
// b (210, 201, 021, 120, 012, 102), t111 the third-order coefficients and L
// = 3 rho u the linear ones, population i is  even_i + odd_i  with
//   even_i = K + 1/2 sec_i(A)
//          = K0 + 1.5 sum_{a: c_a != 0} A_aa + 3 sum_{a<b} c_a c_b A_ab
//   odd_i  = c.L + 1/2 thir_i(B)
//          = c_x X + c_y Y + c_z Z + c_x c_y c_z t111,
//   X = L_x + (3 c_y^2 - 1) b120 + (3 c_z^2 - 1) b102   (Y, Z likewise).
template <typename T>
__host__ __device__ __forceinline__ void eval27(T (&d)[27], T K, const T (&A)[6], const T (&b)[6], T t111, T Lx,
                                                T Ly, T Lz) {
    const T b210 = b[0], b201 = b[1], b021 = b[2], b120 = b[3], b012 = b[4], b102 = b[5];
    // even parts
    const T hx = T(1.5) * A[3], hy = T(1.5) * A[4], hz = T(1.5) * A[5];
    const T txy = T(3) * A[0], txz = T(3) * A[1], tyz = T(3) * A[2];
    const T K0 = fma_(T(-0.5), A[3] + A[4] + A[5], K);
    const T Kx = K0 + hx, Ky = K0 + hy, Kz = K0 + hz;
    const T Exy = Kx + hy, Exz = Kx + hz, Eyz = Ky + hz;
    const T Ec = Exy + hz;
    // odd parts
    const T X00 = Lx - b120 - b102, Y00 = Ly - b210 - b012, Z00 = Lz - b201 - b021;
    const T X10 = fma_(T(3), b120, X00), X01 = fma_(T(3), b102, X00), X11 = fma_(T(3), b102, X10);
    const T Y10 = fma_(T(3), b210, Y00), Y01 = fma_(T(3), b012, Y00), Y11 = fma_(T(3), b012, Y10);
    const T Z10 = fma_(T(3), b201, Z00), Z01 = fma_(T(3), b021, Z00), Z11 = fma_(T(3), b021, Z10);
    T e, o;
    d[0] = K0;
    d[1] = Kx + X00;
    d[3] = Kx - X00;
    d[2] = Ky + Y00;
    d[4] = Ky - Y00;
    d[5] = Kz + Z00;
    d[6] = Kz - Z00;
    e = Exy + txy; o = X10 + Y10; d[7] = e + o; d[9] = e - o;
    e = Exy - txy; o = X10 - Y10; d[10] = e + o; d[8] = e - o;
    e = Exz + txz; o = X01 + Z10; d[11] = e + o; d[17] = e - o;
    e = Exz - txz; o = X01 - Z10; d[15] = e + o; d[13] = e - o;
    e = Eyz + tyz; o = Y01 + Z01; d[12] = e + o; d[18] = e - o;
    e = Eyz - tyz; o = Y01 - Z01; d[16] = e + o; d[14] = e - o;
    const T s = txy + txz, dd = txy - txz, Ep = Ec + tyz, Em = Ec - tyz;
    const T P = X11 + Y11, M = X11 - Y11, Qp = Z11 + t111, R = Z11 - t111;
    e = Ep + s; o = P + Qp; d[19] = e + o; d[25] = e - o;
    e = Em + dd; o = P - Qp; d[23] = e + o; d[21] = e - o;
    e = Em - dd; o = M + R; d[22] = e + o; d[24] = e - o;
    e = Ep - s; o = M - R; d[26] = e + o; d[20] = e - o;
}

// Force-free RR collision (collision.cu:41-119 with F = 0): the populations
// of A = rho a2 + (1 - 1/tau) a2neq and the merged third-order coefficients.
template <typename T>
__host__ __device__ __forceinline__ void collide27(T (&d)[27], const Mom<T> &m, T K, T ux, T uy, T uz,
                                                   T om1) {
    const T rho = T(1) + K;
    T n[6];
    aneq_base(m, rho, ux, uy, uz, n);
    T Aq[6], Bq[10], Bn[10];
    eq_coeffs(rho, ux, uy, uz, Aq, Bq);
    third_from_second(n, ux, uy, uz, om1, Bn);
    T A[6], b[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        A[k] = fma_(om1, n[k], Aq[k]);
        b[k] = Bq[k] + Bn[k];
    }
    eval27(d, K, A, b, Bq[6] + Bn[6], Bq[7], Bq[8], Bq[9]);
}

// Forced RR collision (collision.cu:24-119): with E_i the equilibrium
// deviation (feq_i / w_i - 1) and Fbar_i = 1/2 (c_i - u).F / cs^2, the
// reference's
//   a2neq = sum_i H2_i (f_i + Fbar_i feq_i) - rho u u,
//   f*_i  = feq_i + (1 - 1/tau) fneq_i + Fbar_i feq_i
// become, in deviations, with g_i = (1 + E_i) Fbar_i,
//   a2neq = (the force-free a2neq) + sum_i w_i H2_i g_i,
//   d*_i  = [K + even_i(Aq + (1 - 1/tau) a2neq) + odd_i(Bq + Bn)] + g_i,
// the bracket being the force-free form with the corrected a2neq: two
// evaluations of all populations (E, then the bracket) and the second
// moments of g, instead of a pass over the pairs for the correction and
// another for the populations.
template <typename T>
__host__ __device__ __forceinline__ void collide27_forced(T (&d)[27], const Mom<T> &m, T K, T ux, T uy, T uz,
                                                          T om1, T Fx, T Fy, T Fz) {
    const T rho = T(1) + K;
    T n[6];
    aneq_base(m, rho, ux, uy, uz, n);
    T Aq[6], Bq[10];
    eq_coeffs(rho, ux, uy, uz, Aq, Bq);
    const T bq[6] = {Bq[0], Bq[1], Bq[2], Bq[3], Bq[4], Bq[5]};
    T g[27];
    eval27(g, K, Aq, bq, Bq[6], Bq[7], Bq[8], Bq[9]); // E_i
    // Fbar_i = Fe + 1.5 c_i.F, Fe = -1.5 u.F, by velocity class
    const T Fe = T(-1.5) * fma_(ux, Fx, fma_(uy, Fy, uz * Fz));
    const T fx = T(1.5) * Fx, fy = T(1.5) * Fy, fz = T(1.5) * Fz;
    const T fxyp = fx + fy, fxym = fx - fy, fxzp = fx + fz, fxzm = fx - fz, fyzp = fy + fz, fyzm = fy - fz;
    const T fppp = fxyp + fz, fppm = fxyp - fz, fpmp = fxym + fz, fpmm = fxym - fz;
    T Fo[27];
    Fo[0] = T(0);
    Fo[1] = fx; Fo[3] = -fx; Fo[2] = fy; Fo[4] = -fy; Fo[5] = fz; Fo[6] = -fz;
    Fo[7] = fxyp; Fo[9] = -fxyp; Fo[10] = fxym; Fo[8] = -fxym;
    Fo[11] = fxzp; Fo[17] = -fxzp; Fo[15] = fxzm; Fo[13] = -fxzm;
    Fo[12] = fyzp; Fo[18] = -fyzp; Fo[16] = fyzm; Fo[14] = -fyzm;
    Fo[19] = fppp; Fo[25] = -fppp; Fo[23] = fppm; Fo[21] = -fppm;
    Fo[22] = fpmp; Fo[24] = -fpmp; Fo[26] = fpmm; Fo[20] = -fpmm;
#pragma unroll
    for (int i = 0; i < 27; i++) {
        const T Fb = i == 0 ? Fe : Fe + Fo[i];
        g[i] = fma_(g[i], Fb, Fb); // (1 + E_i) Fbar_i
    }
    // sum_i w_i H2_i g_i: H2_ab = 3 c_a c_b (a != b), 3 c_a^2 - 1
    const Mom<T> mg = moments27(g);
    n[0] = fma_(T(3), mg.pxy, n[0]);
    n[1] = fma_(T(3), mg.pxz, n[1]);
    n[2] = fma_(T(3), mg.pyz, n[2]);
    n[3] = n[3] + fma_(T(3), mg.pxx, -mg.drho);
    n[4] = n[4] + fma_(T(3), mg.pyy, -mg.drho);
    n[5] = n[5] + fma_(T(3), mg.pzz, -mg.drho);
    T Bn[10];
    third_from_second(n, ux, uy, uz, om1, Bn);
    T A[6], b[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        A[k] = fma_(om1, n[k], Aq[k]);
        b[k] = Bq[k] + Bn[k];
    }
    eval27(d, K, A, b, Bq[6] + Bn[6], Bq[7], Bq[8], Bq[9]);
#pragma unroll
    for (int i = 0; i < 27; i++) d[i] = d[i] + g[i];
}

} // namespace rr
