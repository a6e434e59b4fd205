/*
 * rr_oracle.c -- CPU restatement of the reference RR-LBM step (see
 * rr_oracle.h).  TEST INFRASTRUCTURE ONLY: the checker for the CUDA library,
 * never part of the product path.
 *
 * Build with -ffp-contract=off (the Makefile beside this file does), so that
 * the arithmetic is the IEEE sequence written here on x86 and on aarch64.
 */
#include "rr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* lattice tables                                                            */
/* ------------------------------------------------------------------------ */

/* CUDA ordering, RR27V33_code_DNS_LES/initial.cu:67-69 */
static const int CX_CUDA[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1,
                                0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static const int CY_CUDA[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0,
                                -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ_CUDA[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1,
                                1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
/* Fortran ordering, Taylor_Green/D3Q27RR.f90:69-71 == Cavity/para.f90:126-128;
 * its first 19 entries are the D3Q19 set of Taylor_Green/D3Q19RR.f90:75-77 */
static const int CX_F[27] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1,
                             -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1};
static const int CY_F[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0,
                             0, 1, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ_F[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1,
                             -1, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1};

int orc_lattice_init(orc_lattice *L, int q, int order, int cs_mode) {
    if (q != 19 && q != 27) return -1;
    if (q == 19 && order != ORC_ORDER_FORTRAN) return -1; /* D3Q19 exists only in Fortran */
    memset(L, 0, sizeof(*L));
    L->q = q;
    L->ord = order;
    const int *cx = order == ORC_ORDER_CUDA ? CX_CUDA : CX_F;
    const int *cy = order == ORC_ORDER_CUDA ? CY_CUDA : CY_F;
    const int *cz = order == ORC_ORDER_CUDA ? CZ_CUDA : CZ_F;
    for (int i = 0; i < q; i++) {
        L->cx[i] = cx[i];
        L->cy[i] = cy[i];
        L->cz[i] = cz[i];
    }
    for (int i = 0; i < q; i++)
        for (int j = 0; j < q; j++)
            if (cx[j] == -cx[i] && cy[j] == -cy[i] && cz[j] == -cz[i]) L->opp[i] = j;
    /* weights: initial.cu:71-77 (8/27, 2/27, 1/54, 1/216); D3Q19RR.f90:79-81 */
    for (int i = 0; i < q; i++) {
        int n = abs(cx[i]) + abs(cy[i]) + abs(cz[i]);
        if (q == 27)
            L->w[i] = n == 0 ? 8.0 / 27.0 : n == 1 ? 2.0 / 27.0 : n == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
        else
            L->w[i] = n == 0 ? 1.0 / 3.0 : n == 1 ? 1.0 / 18.0 : 1.0 / 36.0;
    }
    /* sound speed: initial.cu:79-81 (cs = sqrt(RT)); D3Q27RR.f90:27-28,84 (cs = 1/sqrt(3)) */
    L->rt = 1.0 / 3.0;
    L->cs = cs_mode == ORC_CS_SQRT_RT ? sqrt(L->rt) : 1.0 / sqrt(3.0);
    L->cs3 = L->rt * L->cs;
    const double cs = L->cs, RT = L->rt, cs3 = L->cs3;
    /* Hermite tables: initial.cu:92-110 == D3Q27RR.f90:114-132 == Cavity/RR.f90:8-30 */
    for (int i = 0; i < q; i++) {
        int x = cx[i], y = cy[i], z = cz[i];
        L->H100[i] = x / cs;
        L->H010[i] = y / cs;
        L->H001[i] = z / cs;
        L->H110[i] = x * y / RT;
        L->H101[i] = x * z / RT;
        L->H011[i] = y * z / RT;
        L->H200[i] = x * x / RT - 1;
        L->H020[i] = y * y / RT - 1;
        L->H002[i] = z * z / RT - 1;
        L->H210[i] = x * x * y / cs3 - y / cs;
        L->H201[i] = x * x * z / cs3 - z / cs;
        L->H021[i] = y * y * z / cs3 - z / cs;
        L->H120[i] = y * y * x / cs3 - x / cs;
        L->H102[i] = z * z * x / cs3 - x / cs;
        L->H012[i] = z * z * y / cs3 - y / cs;
        L->H111[i] = x * y * z / cs3;
        /* D3Q19RR.f90:131-136 */
        L->Hp1[i] = (x * x * y / cs3 - y / cs) + (z * z * y / cs3 - y / cs);
        L->Hm1[i] = (x * x * y / cs3 - y / cs) - (z * z * y / cs3 - y / cs);
        L->Hp2[i] = (z * z * x / cs3 - x / cs) + (y * y * x / cs3 - x / cs);
        L->Hm2[i] = (z * z * x / cs3 - x / cs) - (y * y * x / cs3 - x / cs);
        L->Hp3[i] = (y * y * z / cs3 - z / cs) + (x * x * z / cs3 - z / cs);
        L->Hm3[i] = (y * y * z / cs3 - z / cs) - (x * x * z / cs3 - z / cs);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Hermite projections                                                       */
/* ------------------------------------------------------------------------ */

/* third-order projection with the seven D3Q27 coefficients; the sum order is
 * collision.cu:60-61 for the CUDA ordering and D3Q27RR.f90:345-347 /
 * Cavity/RR.f90:95-97 for the Fortran one.  D3Q19: D3Q19RR.f90:373-378. */
static inline double thir27(const orc_lattice *L, int ip, double a210, double a201, double a021,
                            double a120, double a012, double a102, double a111) {
    if (L->q == 19) {
        double p1 = a210 + a012, p2 = a102 + a120, p3 = a021 + a201;
        double m1 = a210 - a012, m2 = a102 - a120, m3 = a021 - a201;
        return L->Hp1[ip] * p1 + L->Hp2[ip] * p2 + L->Hp3[ip] * p3 + L->Hm1[ip] * m1 / 3.0 +
               L->Hm2[ip] * m2 / 3.0 + L->Hm3[ip] * m3 / 3.0;
    }
    if (L->ord == ORC_ORDER_CUDA)
        return L->H210[ip] * a210 + L->H201[ip] * a201 + L->H021[ip] * a021 + L->H120[ip] * a120 +
               L->H012[ip] * a012 + L->H102[ip] * a102 + 2.0 * L->H111[ip] * a111;
    return L->H210[ip] * a210 + L->H201[ip] * a201 + L->H120[ip] * a120 + L->H021[ip] * a021 +
           L->H102[ip] * a102 + L->H012[ip] * a012 + 2.0 * L->H111[ip] * a111;
}

static inline double sec2(const orc_lattice *L, int ip, double a110, double a101, double a011,
                          double a200, double a020, double a002) {
    return 2.0 * (L->H110[ip] * a110 + L->H101[ip] * a101 + L->H011[ip] * a011) +
           L->H200[ip] * a200 + L->H020[ip] * a020 + L->H002[ip] * a002;
}

/* feqRR: collision.cu:41-69, Cavity/RR.f90:57-107, D3Q27RR.f90:328-349 */
double orc_feq(const orc_lattice *L, int ip, double rho9, double u9, double v9, double w9) {
    double uu = u9 / L->cs, vv = v9 / L->cs, ww = w9 / L->cs;
    double a110 = uu * vv, a101 = uu * ww, a011 = vv * ww, a200 = uu * uu, a020 = vv * vv,
           a002 = ww * ww;
    double a210 = a200 * vv, a201 = a200 * ww, a120 = a020 * uu, a021 = a020 * ww,
           a012 = a002 * vv, a102 = a002 * uu, a111 = a110 * ww;
    double fir = L->H100[ip] * uu + L->H010[ip] * vv + L->H001[ip] * ww;
    double sec = sec2(L, ip, a110, a101, a011, a200, a020, a002);
    double thir = thir27(L, ip, a210, a201, a021, a120, a012, a102, a111);
    return L->w[ip] * rho9 * (1.0 + fir + 0.5 * (sec + thir));
}

/* Non-equilibrium Hermite coefficients from the populations, with the
 * force correction f_i + Fbar_i*feq_i (collision.cu:50-94, BC.cu:39-78,
 * Cavity/RR.f90:110-157).  Fills fbar[] and feq[] as by-products. */
static void aneq(const orc_lattice *L, const double F[3], double rho9, double u9, double v9,
                 double w9, const double *f, double *fbar, double *feq, double ane[13]) {
    const int q = L->q;
    double fx9 = F[0], fy9 = F[1], fz9 = F[2];
    double G3 = u9 * fx9 + v9 * fy9 + w9 * fz9;
    double uu = u9 / L->cs, vv = v9 / L->cs, ww = w9 / L->cs;
    double a110 = uu * vv, a101 = uu * ww, a011 = vv * ww, a200 = uu * uu, a020 = vv * vv,
           a002 = ww * ww;
    double a_110 = rho9 * uu * vv, a_101 = rho9 * uu * ww, a_011 = rho9 * vv * ww;
    double a_200 = rho9 * uu * uu, a_020 = rho9 * vv * vv, a_002 = rho9 * ww * ww;
    double a210 = a200 * vv, a201 = a200 * ww, a120 = a020 * uu, a021 = a020 * ww,
           a012 = a002 * vv, a102 = a002 * uu, a111 = a110 * ww;
    double n110 = 0.0, n101 = 0.0, n011 = 0.0, n200 = 0.0, n020 = 0.0, n002 = 0.0;
    for (int ip = 0; ip < q; ip++) {
        double G1 = L->cx[ip] * fx9 + L->cy[ip] * fy9 + L->cz[ip] * fz9;
        fbar[ip] = 0.5 * (G1 - G3) / L->rt;
        double fir = L->H100[ip] * uu + L->H010[ip] * vv + L->H001[ip] * ww;
        double sec = sec2(L, ip, a110, a101, a011, a200, a020, a002);
        double thir = thir27(L, ip, a210, a201, a021, a120, a012, a102, a111);
        feq[ip] = L->w[ip] * rho9 * (1.0 + fir + 0.5 * (sec + thir));
        double g = f[ip] + fbar[ip] * feq[ip];
        n110 += L->H110[ip] * g;
        n101 += L->H101[ip] * g;
        n011 += L->H011[ip] * g;
        n200 += L->H200[ip] * g;
        n020 += L->H020[ip] * g;
        n002 += L->H002[ip] * g;
    }
    n110 = n110 - a_110;
    n101 = n101 - a_101;
    n011 = n011 - a_011;
    n200 = n200 - a_200;
    n020 = n020 - a_020;
    n002 = n002 - a_002;
    /* recursive third order: collision.cu:88-94 */
    ane[0] = n110;
    ane[1] = n101;
    ane[2] = n011;
    ane[3] = n200;
    ane[4] = n020;
    ane[5] = n002;
    ane[6] = n200 * vv + 2. * uu * n110;  /* 210 */
    ane[7] = n200 * ww + 2. * uu * n101;  /* 201 */
    ane[8] = n020 * uu + 2. * vv * n110;  /* 120 */
    ane[9] = n020 * ww + 2. * vv * n011;  /* 021 */
    ane[10] = n002 * uu + 2. * ww * n101; /* 102 */
    ane[11] = n002 * vv + 2. * ww * n011; /* 012 */
    ane[12] = n110 * ww + n101 * vv + n011 * uu;
}

/* fneqRR_i: collision.cu:106-115 */
static inline double fneq_rr(const orc_lattice *L, int ip, const double ane[13]) {
    double secneq = sec2(L, ip, ane[0], ane[1], ane[2], ane[3], ane[4], ane[5]);
    double thirneq = thir27(L, ip, ane[6], ane[7], ane[9], ane[8], ane[11], ane[10], ane[12]);
    return L->w[ip] * (0.5 * (secneq + thirneq));
}

/* collision_RR, collision.cu:4-120 (== D3Q27RR.f90:319-398 and
 * Cavity/collision.f90:2-49 when the force is zero) */
void orc_collide_node(const orc_lattice *L, double tau_eff, const double F[3], double rho9,
                      double u9, double v9, double w9, double *f) {
    double fbar[27], feq[27], ane[13];
    aneq(L, F, rho9, u9, v9, w9, f, fbar, feq, ane);
    for (int ip = 0; ip < L->q; ip++) {
        double fneq = fneq_rr(L, ip, ane);
        f[ip] = feq[ip] + (1.0 - 1.0 / tau_eff) * fneq + fbar[ip] * feq[ip];
    }
}

/* ------------------------------------------------------------------------ */
/* Taylor-Green program with default-REAL intermediates                      */
/* ------------------------------------------------------------------------ */

/* Hermite tables stored as default REAL (D3Q27RR.f90:57-61, 114-132) */
typedef struct {
    float H100[27], H010[27], H001[27], H110[27], H101[27], H011[27], H200[27], H020[27],
        H002[27], H210[27], H201[27], H021[27], H120[27], H102[27], H012[27], H111[27];
    float Hp1[27], Hm1[27], Hp2[27], Hm2[27], Hp3[27], Hm3[27];
} tab4;

static void tab4_init(const orc_lattice *L, tab4 *T) {
    for (int i = 0; i < L->q; i++) {
        T->H100[i] = (float)L->H100[i];
        T->H010[i] = (float)L->H010[i];
        T->H001[i] = (float)L->H001[i];
        T->H110[i] = (float)L->H110[i];
        T->H101[i] = (float)L->H101[i];
        T->H011[i] = (float)L->H011[i];
        T->H200[i] = (float)L->H200[i];
        T->H020[i] = (float)L->H020[i];
        T->H002[i] = (float)L->H002[i];
        T->H210[i] = (float)L->H210[i];
        T->H201[i] = (float)L->H201[i];
        T->H021[i] = (float)L->H021[i];
        T->H120[i] = (float)L->H120[i];
        T->H102[i] = (float)L->H102[i];
        T->H012[i] = (float)L->H012[i];
        T->H111[i] = (float)L->H111[i];
        T->Hp1[i] = (float)L->Hp1[i];
        T->Hm1[i] = (float)L->Hm1[i];
        T->Hp2[i] = (float)L->Hp2[i];
        T->Hm2[i] = (float)L->Hm2[i];
        T->Hp3[i] = (float)L->Hp3[i];
        T->Hm3[i] = (float)L->Hm3[i];
    }
}

/* sec, single precision: D3Q27RR.f90:343-344 */
static inline float sec4(const tab4 *T, int ip, float a110, float a101, float a011, float a200,
                         float a020, float a002) {
    return 2.0f * (T->H110[ip] * a110 + T->H101[ip] * a101 + T->H011[ip] * a011) +
           T->H200[ip] * a200 + T->H020[ip] * a020 + T->H002[ip] * a002;
}

/* thir, single precision: D3Q27RR.f90:345-347; D3Q19RR.f90:373-378, whose
 * "/ 3.d0" terms are evaluated in double and the sum rounded back */
static inline float thir4(const orc_lattice *L, const tab4 *T, int ip, float a210, float a201,
                          float a021, float a120, float a012, float a102, float a111) {
    if (L->q == 19) {
        float p1 = a210 + a012, p2 = a102 + a120, p3 = a021 + a201;
        float m1 = a210 - a012, m2 = a102 - a120, m3 = a021 - a201;
        float s = T->Hp1[ip] * p1 + T->Hp2[ip] * p2 + T->Hp3[ip] * p3;
        double d = (double)s + (double)(T->Hm1[ip] * m1) / 3.0;
        d = d + (double)(T->Hm2[ip] * m2) / 3.0;
        d = d + (double)(T->Hm3[ip] * m3) / 3.0;
        return (float)d;
    }
    return T->H210[ip] * a210 + T->H201[ip] * a201 + T->H120[ip] * a120 + T->H021[ip] * a021 +
           T->H102[ip] * a102 + T->H012[ip] * a012 + 2.0f * T->H111[ip] * a111;
}

/* collision of D3Q27RR.f90:323-395 with its declared kinds */
static void collide_node_tg4(const orc_lattice *L, const tab4 *T, double tau, double rho9,
                             double u9, double v9, double w9, double *f) {
    double feq9[27];
    float uu = (float)(u9 / L->cs), vv = (float)(v9 / L->cs), ww = (float)(w9 / L->cs);
    float a110 = uu * vv, a101 = uu * ww, a011 = vv * ww, a200 = uu * uu, a020 = vv * vv,
          a002 = ww * ww;
    float a210 = a200 * vv, a201 = a200 * ww, a120 = a020 * uu, a021 = a020 * ww,
          a102 = a002 * uu, a012 = a002 * vv, a111 = a110 * ww;
    for (int ip = 0; ip < L->q; ip++) {
        float eu = T->H100[ip] * uu + T->H010[ip] * vv + T->H001[ip] * ww;
        float sec = sec4(T, ip, a110, a101, a011, a200, a020, a002);
        float thir = thir4(L, T, ip, a210, a201, a021, a120, a012, a102, a111);
        feq9[ip] = (double)(1.0f + eu + 0.5f * (sec + thir));
        feq9[ip] = L->w[ip] * rho9 * feq9[ip];
    }
    a110 = (float)(rho9 * uu * vv);
    a101 = (float)(rho9 * uu * ww);
    a011 = (float)(rho9 * vv * ww);
    a200 = (float)(rho9 * uu * uu);
    a020 = (float)(rho9 * vv * vv);
    a002 = (float)(rho9 * ww * ww);
    float n110 = 0.0f, n101 = 0.0f, n011 = 0.0f, n200 = 0.0f, n020 = 0.0f, n002 = 0.0f;
    for (int ip = 0; ip < L->q; ip++) {
        double f9 = f[ip];
        n110 = (float)(n110 + T->H110[ip] * f9);
        n101 = (float)(n101 + T->H101[ip] * f9);
        n011 = (float)(n011 + T->H011[ip] * f9);
        n200 = (float)(n200 + T->H200[ip] * f9);
        n020 = (float)(n020 + T->H020[ip] * f9);
        n002 = (float)(n002 + T->H002[ip] * f9);
    }
    n110 = n110 - a110;
    n101 = n101 - a101;
    n011 = n011 - a011;
    n200 = n200 - a200;
    n020 = n020 - a020;
    n002 = n002 - a002;
    float n210 = n200 * vv + 2.0f * uu * n110, n201 = n200 * ww + 2.0f * uu * n101;
    float n120 = n020 * uu + 2.0f * vv * n110, n021 = n020 * ww + 2.0f * vv * n011;
    float n102 = n002 * uu + 2.0f * ww * n101, n012 = n002 * vv + 2.0f * ww * n011;
    float n111 = n110 * ww + n101 * vv + n011 * uu;
    for (int ip = 0; ip < L->q; ip++) {
        float sec = sec4(T, ip, n110, n101, n011, n200, n020, n002);
        float thir = thir4(L, T, ip, n210, n201, n021, n120, n012, n102, n111);
        double fneq9 = L->w[ip] * 0.5 * (double)(sec + thir);
        f[ip] = feq9[ip] + (1.0 - 1.0 / tau) * fneq9;
    }
}

/* macrovar, macrovar.cu:4-31 (Cavity/collision.f90:51-89, D3Q27RR.f90:421-437) */
void orc_moments_node(const orc_lattice *L, const double F[3], const double *f, double *rho,
                      double *u, double *v, double *w) {
    double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
    for (int ip = 0; ip < L->q; ip++) {
        double fv = f[ip];
        r += fv;
        jx += L->cx[ip] * fv;
        jy += L->cy[ip] * fv;
        jz += L->cz[ip] * fv;
    }
    *rho = r;
    *u = (jx + 0.5 * F[0]) / r;
    *v = (jy + 0.5 * F[1]) / r;
    *w = (jz + 0.5 * F[2]) / r;
}

/* regularized wall closure: RRBC BC.cu:4-126 == Cavity/streaming.f90:103-137.
 * Rebuilds the populations flagged in entering[] from the node's moments. */
void orc_regularize_node(const orc_lattice *L, const double F[3], double *f,
                         const int *entering) {
    double rho9, u9, v9, w9, fbar[27], feq[27], ane[13];
    orc_moments_node(L, F, f, &rho9, &u9, &v9, &w9);
    aneq(L, F, rho9, u9, v9, w9, f, fbar, feq, ane);
    for (int ip = 0; ip < L->q; ip++) {
        if (!entering[ip]) continue;
        double fneq = fneq_rr(L, ip, ane);
        f[ip] = feq[ip] + fneq - fbar[ip] * feq[ip];
    }
}

/* ------------------------------------------------------------------------ */
/* whole-grid routines                                                       */
/* ------------------------------------------------------------------------ */

static inline int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

/* the body force at node idx: the per-node field when there is one */
static inline void node_force(const orc_params *P, long N, long idx, double F[3]) {
    if (P->ffield) {
        F[0] = P->ffield[idx];
        F[1] = P->ffield[N + idx];
        F[2] = P->ffield[2 * N + idx];
    } else {
        F[0] = P->force[0];
        F[1] = P->force[1];
        F[2] = P->force[2];
    }
}

/* stream (pull form of streaming.cu:3-24 / D3Q27RR.f90:400-419), then the wall
 * faces in the order x-lo, x-hi, y-lo, y-hi, z-lo, z-hi: half-way bounce-back
 * from the post-collision value of the opposite population at the same node
 * (BB streaming.cu:26-56, Cavity/streaming.f90:91-99) with the moving-wall
 * term +6 w_i (c_i . U_wall) (Cavity/streaming.f90:142-152), then the
 * regularized closure of the entering populations
 * (Cavity/streaming.f90:100-140; BC.cu:4-126 after macrovar). */
void orc_stream_walls(const orc_params *P, const double *fin, double *fout) {
    const orc_lattice *L = &P->lat;
    const int nx = P->nx, ny = P->ny, nz = P->nz, q = L->q;
    const long N = (long)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++) {
        double fl[27];
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                long idx = ((long)z * ny + y) * nx + x;
                for (int ip = 0; ip < q; ip++) {
                    int xs = wrapi(x - L->cx[ip], nx), ys = wrapi(y - L->cy[ip], ny),
                        zs = wrapi(z - L->cz[ip], nz);
                    fl[ip] = fin[ip * N + ((long)zs * ny + ys) * nx + xs];
                }
                int on[6] = {x == 0, x == nx - 1, y == 0, y == ny - 1, z == 0, z == nz - 1};
                for (int face = 0; face < 6; face++) {
                    if (P->face[face] == ORC_FACE_PERIODIC || !on[face]) continue;
                    int axis = face / 2, sgn = (face % 2 == 0) ? 1 : -1; /* inward normal */
                    int entering[27];
                    const double *U = P->uwall[face];
                    for (int ip = 0; ip < q; ip++) {
                        int c = axis == 0 ? L->cx[ip] : axis == 1 ? L->cy[ip] : L->cz[ip];
                        entering[ip] = (c * sgn > 0);
                        if (!entering[ip]) continue;
                        double v = fin[L->opp[ip] * N + idx];
                        if (U[0] != 0.0 || U[1] != 0.0 || U[2] != 0.0) {
                            double cu = L->cx[ip] * U[0] + L->cy[ip] * U[1] + L->cz[ip] * U[2];
                            v = v + 6. * L->w[ip] * cu;
                        }
                        fl[ip] = v;
                    }
                    if (P->face[face] == ORC_FACE_WALL) {
                        double Fn[3];
                        node_force(P, N, idx, Fn);
                        orc_regularize_node(L, Fn, fl, entering);
                    }
                }
                for (int ip = 0; ip < q; ip++) fout[ip * N + idx] = fl[ip];
            }
    }
}

void orc_moments_all(const orc_params *P, const double *f, double *rho, double *ux, double *uy,
                     double *uz) {
    const orc_lattice *L = &P->lat;
    const long N = (long)P->nx * P->ny * P->nz;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < N; idx++) {
        double fl[27];
        for (int ip = 0; ip < L->q; ip++) fl[ip] = f[ip * N + idx];
        double Fn[3];
        node_force(P, N, idx, Fn);
        if (P->bgk) {
            /* BGK/macrovar.cu:16-30: rho = sum f, u = sum c f + F/2 */
            double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
            for (int ip = 0; ip < L->q; ip++) {
                r += fl[ip];
                jx += L->cx[ip] * fl[ip];
                jy += L->cy[ip] * fl[ip];
                jz += L->cz[ip] * fl[ip];
            }
            rho[idx] = r;
            ux[idx] = jx + 0.5 * Fn[0];
            uy[idx] = jy + 0.5 * Fn[1];
            uz[idx] = jz + 0.5 * Fn[2];
        } else {
            orc_moments_node(L, Fn, fl, &rho[idx], &ux[idx], &uy[idx], &uz[idx]);
        }
    }
}

/* BGK/collision.cu:11-33: feq = w (rho + eu + (eu^2 - uv) / 2) with
 * eu = c.u / RT, uv = u.u / RT; f += -(f - feq) / tau + (1 - 0.5 / tau)
 * (c.F - u.F) / RT w (1 + eu + (eu^2 - uv) / 2) */
void orc_bgk_node(const orc_lattice *L, double tau, const double F[3], double rho9, double u9, double v9,
                  double w9, double *f) {
    const double fx9 = F[0], fy9 = F[1], fz9 = F[2];
    const double G3 = u9 * fx9 + v9 * fy9 + w9 * fz9;
    for (int ip = 0; ip < L->q; ip++) {
        const double RT = 1.0 / 3.0;
        const double eu = (L->cx[ip] * u9 + L->cy[ip] * v9 + L->cz[ip] * w9) / RT;
        const double uv = (u9 * u9 + v9 * v9 + w9 * w9) / RT;
        const double feq = L->w[ip] * (rho9 + eu + 0.5 * (eu * eu - uv));
        const double G1 = L->cx[ip] * fx9 + L->cy[ip] * fy9 + L->cz[ip] * fz9;
        double fchange = -(f[ip] - feq) / tau;
        const double feq_rho0 = L->w[ip] * (1.0 + eu + 0.5 * (eu * eu - uv));
        fchange += (1.0 - 0.5 / tau) * (G1 - G3) / RT * feq_rho0;
        f[ip] += fchange;
    }
}

void orc_collide_all(const orc_params *P, double *f, const double *rho, const double *ux,
                     const double *uy, const double *uz, const double *taut) {
    const orc_lattice *L = &P->lat;
    const long N = (long)P->nx * P->ny * P->nz;
    tab4 T;
    if (P->tg_real4) tab4_init(L, &T);
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < N; idx++) {
        double fl[27];
        for (int ip = 0; ip < L->q; ip++) fl[ip] = f[ip * N + idx];
        /* collision.cu:27-31 */
        double tau_eff = P->les ? P->tau + taut[idx] : P->tau;
        if (P->bgk) {
            double Fn[3];
            node_force(P, N, idx, Fn);
            orc_bgk_node(L, P->tau, Fn, rho[idx], ux[idx], uy[idx], uz[idx], fl);
        } else if (P->tg_real4)
            collide_node_tg4(L, &T, tau_eff, rho[idx], ux[idx], uy[idx], uz[idx], fl);
        else {
            double Fn[3];
            node_force(P, N, idx, Fn);
            orc_collide_node(L, tau_eff, Fn, rho[idx], ux[idx], uy[idx], uz[idx], fl);
        }
        for (int ip = 0; ip < L->q; ip++) f[ip * N + idx] = fl[ip];
    }
}

/* WALE, LES.cu:4-98.  The reference has walls only at y = 0 and y = LY-1 and
 * central differences elsewhere; here any face flagged as a wall gets the
 * reference's one-sided wall formula (LES.cu:19-28) along its axis.  The one
 * deviation: S:S = Sd:Sd = 0 gives 0 instead of the reference's 0/0 = NaN. */
void orc_wale(const orc_params *P, const double *ux, const double *uy, const double *uz,
              double *taut) {
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const double cw = P->cw;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                long idx = ((long)iz * ny + iy) * nx + ix;
                double g[3][3]; /* g[a][b] = d u_a / d x_b */
                const double *U[3] = {ux, uy, uz};
                int pos[3] = {ix, iy, iz}, n[3] = {nx, ny, nz};
                long stride[3] = {1, nx, (long)nx * ny};
                for (int b = 0; b < 3; b++) {
                    int lo_wall = P->face[2 * b] != ORC_FACE_PERIODIC;
                    int hi_wall = P->face[2 * b + 1] != ORC_FACE_PERIODIC;
                    int p = pos[b];
                    for (int a = 0; a < 3; a++) {
                        const double *u = U[a];
                        if (p == 0 && lo_wall) {
                            long ip1 = idx + stride[b];
                            g[a][b] = (3.0 * u[idx] + u[ip1]) / 3.0;
                        } else if (p == n[b] - 1 && hi_wall) {
                            long im1 = idx - stride[b];
                            g[a][b] = (-3.0 * u[idx] - u[im1]) / 3.0;
                        } else {
                            long ip1 = p == n[b] - 1 ? idx - (long)(n[b] - 1) * stride[b] : idx + stride[b];
                            long im1 = p == 0 ? idx + (long)(n[b] - 1) * stride[b] : idx - stride[b];
                            g[a][b] = 0.5 * (u[ip1] - u[im1]);
                        }
                    }
                }
                double dudx = g[0][0], dudy = g[0][1], dudz = g[0][2];
                double dvdx = g[1][0], dvdy = g[1][1], dvdz = g[1][2];
                double dwdx = g[2][0], dwdy = g[2][1], dwdz = g[2][2];
                /* LES.cu:79-97 */
                double sijsq = (dudy + dvdx) * (dudy + dvdx) + (dudz + dwdx) * (dudz + dwdx) +
                               (dvdz + dwdy) * (dvdz + dwdy);
                sijsq = 0.5 * sijsq + dudx * dudx + dvdy * dvdy + dwdz * dwdz;
                double s11d = 2. * dudx * dudx - dvdy * dvdy - dwdz * dwdz + dudy * dvdx +
                              dudz * dwdx - 2. * dvdz * dwdy;
                s11d = s11d / 3.;
                double s12d = dudx * (dudy + dvdx) + dudy * dvdy + dvdx * dvdy + dvdz * dwdx +
                              dudz * dwdy;
                s12d = 0.5 * s12d;
                double s13d = dudx * (dudz + dwdx) + dudy * dvdz + dvdx * dwdy + dudz * dwdz +
                              dwdx * dwdz;
                s13d = 0.5 * s13d;
                double s22d = 2. * dvdy * dvdy - dudx * dudx - dwdz * dwdz + dudy * dvdx +
                              dvdz * dwdy - 2. * dudz * dwdx;
                s22d = s22d / 3.;
                double s23d = dvdy * (dvdz + dwdy) + dudz * dvdx + dudy * dwdx + dvdz * dwdz +
                              dwdy * dwdz;
                s23d = 0.5 * s23d;
                double s33d = 2. * dwdz * dwdz - dudx * dudx - dvdy * dvdy + dudz * dwdx +
                              dvdz * dwdy - 2. * dudy * dvdx;
                s33d = s33d / 3.;
                double sijdsq = s11d * s11d + s22d * s22d + s33d * s33d +
                                2.0 * (s12d * s12d + s13d * s13d + s23d * s23d);
                double den = pow(sijsq, 2.5) + pow(sijdsq, 1.25);
                taut[idx] = den > 0.0 ? 3.0 * cw * cw * pow(sijdsq, 1.5) / den : 0.0;
            }
}

void orc_fdbc(const orc_params *P, double *f, double *rho, double *ux, double *uy, double *uz,
              const double *taut) {
    const orc_lattice *L = &P->lat;
    const int nx = P->nx, ny = P->ny, nz = P->nz, q = L->q;
    const long N = (long)nx * ny * nz;
    /* (1) wall velocity from the first two rows inside: the quadratic through
     * u = 0 on the wall half a node out, u(1) and u(2), at the wall node */
    for (int side = 0; side < 2; side++) {
        if (P->face[2 + side] != ORC_FACE_FDBC) continue;
        const int iy = side ? ny - 1 : 0, dy = side ? -1 : 1;
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                const long idx = ((long)iz * ny + iy) * nx + ix;
                const long i1 = ((long)iz * ny + iy + dy) * nx + ix, i2 = ((long)iz * ny + iy + 2 * dy) * nx + ix;
                ux[idx] = 2.0 / 3.0 * ux[i1] - 1.0 / 5.0 * ux[i2];
                uy[idx] = 2.0 / 3.0 * uy[i1] - 1.0 / 5.0 * uy[i2];
                uz[idx] = 2.0 / 3.0 * uz[i1] - 1.0 / 5.0 * uz[i2];
            }
    }
    /* (2) the closure, BC.cu:162-308 */
    for (int side = 0; side < 2; side++) {
        if (P->face[2 + side] != ORC_FACE_FDBC) continue;
        const int iy = side ? ny - 1 : 0;
#pragma omp parallel for schedule(static)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                const long idx = ((long)iz * ny + iy) * nx + ix;
                const double tau_eff = taut ? P->tau + taut[idx] : P->tau;
                double dudy, dvdy, dwdy;
                if (!side) {
                    const long p1 = ((long)iz * ny + iy + 1) * nx + ix, p2 = ((long)iz * ny + iy + 2) * nx + ix;
                    dudy = (-3.0 * ux[idx] + 4.0 * ux[p1] - ux[p2]) / 2.0;
                    dvdy = (-3.0 * uy[idx] + 4.0 * uy[p1] - uy[p2]) / 2.0;
                    dwdy = (-3.0 * uz[idx] + 4.0 * uz[p1] - uz[p2]) / 2.0;
                } else {
                    const long m1 = ((long)iz * ny + iy - 1) * nx + ix, m2 = ((long)iz * ny + iy - 2) * nx + ix;
                    dudy = (3.0 * ux[idx] - 4.0 * ux[m1] + ux[m2]) / 2.0;
                    dvdy = (3.0 * uy[idx] - 4.0 * uy[m1] + uy[m2]) / 2.0;
                    dwdy = (3.0 * uz[idx] - 4.0 * uz[m1] + uz[m2]) / 2.0;
                }
                const int ixp = (ix + 1) % nx, ixm = (ix - 1 + nx) % nx;
                const int izp = (iz + 1) % nz, izm = (iz - 1 + nz) % nz;
                const long xp = ((long)iz * ny + iy) * nx + ixp, xm = ((long)iz * ny + iy) * nx + ixm;
                const long zp = ((long)izp * ny + iy) * nx + ix, zm = ((long)izm * ny + iy) * nx + ix;
                const double dudx = 0.5 * (ux[xp] - ux[xm]), dvdx = 0.5 * (uy[xp] - uy[xm]),
                             dwdx = 0.5 * (uz[xp] - uz[xm]);
                const double dudz = 0.5 * (ux[zp] - ux[zm]), dvdz = 0.5 * (uy[zp] - uy[zm]),
                             dwdz = 0.5 * (uz[zp] - uz[zm]);
                const double S110 = 0.5 * (dudy + dvdx), S101 = 0.5 * (dudz + dwdx), S011 = 0.5 * (dvdz + dwdy);
                const double S200 = dudx, S020 = dvdy, S002 = dwdz;
                double F[3];
                node_force(P, N, idx, F);
                const double fx9 = F[0], fy9 = F[1], fz9 = F[2];
                const double u9 = ux[idx], v9 = uy[idx], w9 = uz[idx];
                const double G3 = u9 * fx9 + v9 * fy9 + w9 * fz9;
                const double uu = u9 / L->cs, vv = v9 / L->cs, ww = w9 / L->cs;
                const double a110 = uu * vv, a101 = uu * ww, a011 = vv * ww, a200 = uu * uu, a020 = vv * vv,
                             a002 = ww * ww;
                const double a210 = a200 * vv, a201 = a200 * ww, a120 = a020 * uu, a021 = a020 * ww,
                             a012 = a002 * vv, a102 = a002 * uu, a111 = a110 * ww;
                double fbar[27], fir[27], sec[27], thir[27];
                for (int ip = 0; ip < q; ip++) {
                    const double G1 = L->cx[ip] * fx9 + L->cy[ip] * fy9 + L->cz[ip] * fz9;
                    fbar[ip] = 0.5 * (G1 - G3) / L->rt;
                    fir[ip] = L->H100[ip] * uu + L->H010[ip] * vv + L->H001[ip] * ww;
                    sec[ip] = sec2(L, ip, a110, a101, a011, a200, a020, a002);
                    thir[ip] = thir27(L, ip, a210, a201, a021, a120, a012, a102, a111);
                }
                /* the non-equilibrium coefficients -rho tau S and their
                 * recursive third order (BC.cu:227-241, 265-279) */
                double ane[13];
                double rho9 = 1.0; /* BC.cu:213: the density the known-population balance starts from */
                double sum_f_ps = 0.0, sum_g_in = 0.0;
                for (int pass = 0; pass < 2; pass++) {
                    ane[0] = -rho9 * tau_eff * S110;
                    ane[1] = -rho9 * tau_eff * S101;
                    ane[2] = -rho9 * tau_eff * S011;
                    ane[3] = -rho9 * tau_eff * S200;
                    ane[4] = -rho9 * tau_eff * S020;
                    ane[5] = -rho9 * tau_eff * S002;
                    ane[6] = ane[3] * vv + 2. * uu * ane[0];  /* 210 */
                    ane[7] = ane[3] * ww + 2. * uu * ane[1];  /* 201 */
                    ane[8] = ane[4] * uu + 2. * vv * ane[0];  /* 120 */
                    ane[9] = ane[4] * ww + 2. * vv * ane[2];  /* 021 */
                    ane[10] = ane[5] * uu + 2. * ww * ane[1]; /* 102 */
                    ane[11] = ane[5] * vv + 2. * ww * ane[2]; /* 012 */
                    ane[12] = ane[0] * ww + ane[1] * vv + ane[2] * uu;
                    for (int ip = 0; ip < q; ip++) {
                        /* known: the populations streamed in from inside (BC.cu:245) */
                        const int known = side ? (L->cy[ip] > 0) : (L->cy[ip] < 0);
                        if (pass == 0 && !known) continue;
                        const double feq = L->w[ip] * rho9 * (1.0 + fir[ip] + 0.5 * (sec[ip] + thir[ip]));
                        const double secneq = sec2(L, ip, ane[0], ane[1], ane[2], ane[3], ane[4], ane[5]);
                        const double thirneq = thir27(L, ip, ane[6], ane[7], ane[9], ane[8], ane[11], ane[10], ane[12]);
                        const double fneq = L->w[ip] * (secneq + thirneq);
                        const double g = feq + fneq - fbar[ip] * feq;
                        if (pass == 0) {
                            sum_f_ps += f[ip * N + idx];
                            sum_g_in += g;
                        } else {
                            f[ip * N + idx] = g;
                        }
                    }
                    /* BC.cu:262: the density that balances the known populations */
                    if (pass == 0) rho9 = sum_f_ps / sum_g_in;
                }
            }
    }
    /* (3) macrovar_BN */
    for (int side = 0; side < 2; side++) {
        if (P->face[2 + side] != ORC_FACE_FDBC) continue;
        const int iy = side ? ny - 1 : 0;
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                const long idx = ((long)iz * ny + iy) * nx + ix;
                double fl[27], F[3];
                for (int ip = 0; ip < q; ip++) fl[ip] = f[ip * N + idx];
                node_force(P, N, idx, F);
                orc_moments_node(L, F, fl, &rho[idx], &ux[idx], &uy[idx], &uz[idx]);
            }
    }
}

/* one reference time step, main.cu:373-409: [WALE] -> collide -> stream+BB
 * -> moments -> wall closure -> wall moments.  The wall closure is folded
 * into orc_stream_walls (it only needs the node's own populations), and the
 * final moments pass covers the wall nodes too (macrovar_BN). */
void orc_step(const orc_params *P, orc_state *S) {
    if (P->les) orc_wale(P, S->ux, S->uy, S->uz, S->taut);
    orc_collide_all(P, S->f, S->rho, S->ux, S->uy, S->uz, S->taut);
    orc_stream_walls(P, S->f, S->ftmp);
    double *t = S->f;
    S->f = S->ftmp;
    S->ftmp = t;
    orc_moments_all(P, S->f, S->rho, S->ux, S->uy, S->uz);
    if (P->face[2] == ORC_FACE_FDBC || P->face[3] == ORC_FACE_FDBC)
        orc_fdbc(P, S->f, S->rho, S->ux, S->uy, S->uz, P->les ? S->taut : NULL);
}

void orc_run(const orc_params *P, orc_state *S, int nsteps) {
    for (int i = 0; i < nsteps; i++) orc_step(P, S);
}

void orc_srand(orc_trip *T, unsigned seed) {
    int32_t r[344];
    r[0] = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
        long long w = (16807LL * (long long)r[i - 1]) % 2147483647LL;
        if (w < 0) w += 2147483647LL;
        r[i] = (int32_t)w;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 34; i < 344; i++) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
    for (int i = 0; i < 34; i++) T->r[i] = r[310 + i];
    T->k = 0; /* r[k] holds term i - 34 of the next term i */
}

int orc_rand(orc_trip *T) {
    /* ring of the last 34 terms: oldest at k; term i-31 is at k+3, i-3 at k+31 */
    const int32_t v = (int32_t)((uint32_t)T->r[(T->k + 3) % 34] + (uint32_t)T->r[(T->k + 31) % 34]);
    T->r[T->k] = v;
    T->k = (T->k + 1) % 34;
    return (int)((uint32_t)v >> 1);
}

/* forcing_GP of macrovar.cu:76-115, written in the same operation order so
 * that it rounds as the reference does (integer divisions included:
 * LY / 4, and ix / LX, which is 0 inside the domain) */
void orc_trip_force(const orc_params *P, long long n, double phase, double *fx, double *fy, double *fz) {
    const int LX = P->nx, LY = P->ny, LZ = P->nz;
    const double pi2 = 2 * acos(-1.0);
    const double Tpd = 2000.0;
    const double LYq = LY / 4;
    const int h0 = 2;
    const double beta9 = 3.0, gamma9 = 2.0;
    const double F0 = P->force[0];
    const double Amp0 = (100.0 * beta9 / LY) * sin(pi2 * (double)n / Tpd);
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < LZ; iz++)
        for (int iy = 0; iy < LY; iy++)
            for (int ix = 0; ix < LX; ix++) {
                const long idx = ((long)iz * LY + iy) * LX + ix;
                double x = F0, y = 0.0, z = 0.0;
                if (iy > h0 && iy < LYq + h0) {
                    x = F0 * (1.0 - Amp0 * LX / beta9 * sin(pi2 * (iy - h0) / LYq) * sin(beta9 * pi2 * ix / LX) *
                                        cos(gamma9 * pi2 * iz / LZ));
                    y = F0 * Amp0 * 0.5 * LYq * (1 - cos(pi2 * (iy - h0) / LYq)) * cos(beta9 * pi2 * ix / LX) *
                        cos(gamma9 * pi2 * iz / LZ);
                    z = F0 * Amp0 * 0.5 * LZ / gamma9 * sin(pi2 * (iy - h0) / LYq) * cos(beta9 * pi2 * ix / LX) *
                        sin(gamma9 * pi2 * iz / LZ);
                } else if (iy > 0.75 * LY - h0 && iy < LY - h0) {
                    x = F0 * (1.0 + Amp0 * LX / beta9 * sin(pi2 * (-LY + iy + h0 + LYq) / LYq) *
                                        sin(beta9 * pi2 * (ix / LX + phase)) * cos(gamma9 * pi2 * iz / LZ));
                    y = -F0 * Amp0 * 0.5 * LYq * (1 - cos(pi2 * (-LY + iy + h0 + LYq) / LYq)) *
                        cos(beta9 * pi2 * (ix / LX + phase)) * cos(gamma9 * pi2 * iz / LZ);
                    z = -F0 * Amp0 * 0.5 * LZ / gamma9 * sin(pi2 * (-LY + iy + h0 + LYq) / LYq) *
                        cos(beta9 * pi2 * (ix / LX + phase)) * sin(gamma9 * pi2 * iz / LZ);
                }
                fx[idx] = x;
                fy[idx] = y;
                fz[idx] = z;
            }
}

void orc_run_trip(const orc_params *P, orc_state *S, orc_trip *T, int nsteps) {
    const long N = (long)P->nx * P->ny * P->nz;
    orc_params Q = *P;
    for (int i = 0; i < nsteps; i++) {
        const long long n = T->istep + 1;
        if (n < T->trip_steps) {
            if (n % 2000 == 0) T->phase = (double)orc_rand(T) / 2147483647.0;
            orc_trip_force(P, n, T->phase, T->fx, T->fy, T->fz);
        } else {
            for (long idx = 0; idx < N; idx++) {
                T->fx[idx] = P->force[0];
                T->fy[idx] = 0.0;
                T->fz[idx] = 0.0;
            }
        }
        /* the field is contiguous: fx, fy, fz of length N each */
        Q.ffield = T->fx;
        orc_step(&Q, S);
        T->istep = n;
    }
}

/* ------------------------------------------------------------------------ */
/* initial states                                                            */
/* ------------------------------------------------------------------------ */

/* start-state node of D3Q27RR.f90:183-260 with its declared kinds */
static void tg_fill_node4(const orc_lattice *L, const tab4 *T, double tau, double rho9, double u9,
                          double v9, double w9, double dudx, double dudy, double dvdx,
                          double dvdy, double *f, long N, long idx) {
    float uu = (float)(u9 / L->cs), vv = (float)(v9 / L->cs), ww = (float)(w9 / L->cs);
    float a110 = uu * vv, a101 = uu * ww, a011 = vv * ww, a200 = uu * uu, a020 = vv * vv,
          a002 = ww * ww;
    float a210 = a200 * vv, a201 = a200 * ww, a120 = a020 * uu, a021 = a020 * ww,
          a102 = a002 * uu, a012 = a002 * vv, a111 = a110 * ww;
    float n110 = (float)(-tau * rho9 * (dudy + dvdx)), n101 = 0.0f, n011 = 0.0f;
    float n200 = (float)(-tau * rho9 * 2.0 * dudx), n020 = (float)(-tau * rho9 * 2.0 * dvdy);
    float n002 = 0.0f;
    float n210 = n200 * vv + 2.0f * uu * n110, n201 = n200 * ww + 2.0f * uu * n101;
    float n120 = n020 * uu + 2.0f * vv * n110, n021 = n020 * ww + 2.0f * vv * n011;
    float n102 = n002 * uu + 2.0f * ww * n101, n012 = n002 * vv + 2.0f * ww * n011;
    float n111 = n110 * ww + n101 * vv + n011 * uu;
    for (int ip = 0; ip < L->q; ip++) {
        float eu = T->H100[ip] * uu + T->H010[ip] * vv + T->H001[ip] * ww;
        float sec = sec4(T, ip, a110, a101, a011, a200, a020, a002);
        float thir = thir4(L, T, ip, a210, a201, a021, a120, a012, a102, a111);
        double feq9 = (double)(1.0f + eu + 0.5f * (sec + thir));
        feq9 = L->w[ip] * rho9 * feq9;
        float secn = sec4(T, ip, n110, n101, n011, n200, n020, n002);
        float thirn = thir4(L, T, ip, n210, n201, n021, n120, n012, n102, n111);
        double fneq9 = L->w[ip] * 0.5 * (double)(secn + thirn);
        f[ip * N + idx] = feq9 + fneq9;
    }
}

/* Taylor-Green start of Taylor_Green/D3Q27RR.f90:134-264: cell-centred
 * analytic u, v, rho; f = feqRR + fneqRR with the non-equilibrium moments
 * from 4th-order periodic finite differences of u, v. */
static void tg_fill(const orc_params *P, double *f, const double *rho, const double *ux,
                    const double *uy, const double *uz) {
    const orc_lattice *L = &P->lat;
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const long N = (long)nx * ny * nz;
    const double tau = P->tau;
    tab4 T;
    if (P->tg_real4) tab4_init(L, &T);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                long idx = ((long)k * ny + j) * nx + i;
                int ip1 = (i + 1) % nx, ip2 = (i + 2) % nx, im1 = (i - 1 + nx) % nx,
                    im2 = (i - 2 + nx) % nx;
                int jp1 = (j + 1) % ny, jp2 = (j + 2) % ny, jm1 = (j - 1 + ny) % ny,
                    jm2 = (j - 2 + ny) % ny;
#define U_(a, b) ux[((long)k * ny + (b)) * nx + (a)]
#define V_(a, b) uy[((long)k * ny + (b)) * nx + (a)]
                /* D3Q27RR.f90:198-201 */
                double dudx = -(U_(ip2, j) - 8.0 * U_(ip1, j) + 8.0 * U_(im1, j) - U_(im2, j)) / 12.0;
                double dudy = -(U_(i, jp2) - 8.0 * U_(i, jp1) + 8.0 * U_(i, jm1) - U_(i, jm2)) / 12.0;
                double dvdx = -(V_(ip2, j) - 8.0 * V_(ip1, j) + 8.0 * V_(im1, j) - V_(im2, j)) / 12.0;
                double dvdy = -(V_(i, jp2) - 8.0 * V_(i, jp1) + 8.0 * V_(i, jm1) - V_(i, jm2)) / 12.0;
#undef U_
#undef V_
                double rho9 = rho[idx], u9 = ux[idx], v9 = uy[idx], w9 = uz[idx];
                double uu = u9 / L->cs, vv = v9 / L->cs, ww = w9 / L->cs;
                /* D3Q27RR.f90:237-249 */
                double ane[13];
                ane[0] = -tau * rho9 * (dudy + dvdx);
                ane[1] = 0.0;
                ane[2] = 0.0;
                ane[3] = -tau * rho9 * 2.0 * dudx;
                ane[4] = -tau * rho9 * 2.0 * dvdy;
                ane[5] = 0.0;
                ane[6] = ane[3] * vv + 2. * uu * ane[0];
                ane[7] = ane[3] * ww + 2. * uu * ane[1];
                ane[8] = ane[4] * uu + 2. * vv * ane[0];
                ane[9] = ane[4] * ww + 2. * vv * ane[2];
                ane[10] = ane[5] * uu + 2. * ww * ane[1];
                ane[11] = ane[5] * vv + 2. * ww * ane[2];
                ane[12] = ane[0] * ww + ane[1] * vv + ane[2] * uu;
                if (P->tg_real4) {
                    tg_fill_node4(L, &T, tau, rho9, u9, v9, w9, dudx, dudy, dvdx, dvdy, f, N, idx);
                    continue;
                }
                for (int ip = 0; ip < L->q; ip++) {
                    double feq9 = orc_feq(L, ip, rho9, u9, v9, w9);
                    /* D3Q27RR.f90:253-260: wwp9*0.5*(sec+thir) */
                    double secneq = sec2(L, ip, ane[0], ane[1], ane[2], ane[3], ane[4], ane[5]);
                    double thirneq =
                        thir27(L, ip, ane[6], ane[7], ane[9], ane[8], ane[11], ane[10], ane[12]);
                    double fneq9 = L->w[ip] * 0.5 * (secneq + thirneq);
                    f[ip * N + idx] = feq9 + fneq9;
                }
            }
}

/* D3Q27RR.f90:134-146 with k_val = 2 and x = i - 0.5 (1-based i) */
void orc_init_tg_reference(const orc_params *P, double U0, double *f, double *rho, double *ux,
                           double *uy, double *uz) {
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const double pi = 3.14159265358979323846, kv = 2.0, L = nx, cs2 = P->lat.rt;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                long idx = ((long)k * ny + j) * nx + i;
                double x = (double)(float)(i + 1 - 0.5f), y = (double)(float)(j + 1 - 0.5f);
                ux[idx] = -U0 * cos(kv * pi * x / L) * sin(kv * pi * y / L);
                uy[idx] = U0 * cos(kv * pi * y / L) * sin(kv * pi * x / L);
                uz[idx] = 0.0;
                rho[idx] = 1.0 - U0 * U0 / 2 * cos(kv * pi / L * (x - y)) * cos(kv * pi / L * (x + y)) / cs2;
            }
    tg_fill(P, f, rho, ux, uy, uz);
}

/* Taylor-Green start of the 100x100x4 workload: x = ix + 0.5 (0-based),
 * u = U0 sin(2 pi x/L) cos(2 pi y/L), v = -U0 cos(2 pi x/L) sin(2 pi y/L),
 * rho = 1 + 3 p', p' = -(U0^2/4)(cos(4 pi x/L) + cos(4 pi y/L)); f from the
 * same feq + FD-strain fneq construction as the reference start. */
void orc_init_tg_config(const orc_params *P, double U0, double *f, double *rho, double *ux,
                        double *uy, double *uz) {
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const double pi = 3.14159265358979323846, L = nx;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                long idx = ((long)k * ny + j) * nx + i;
                double x = i + 0.5, y = j + 0.5;
                ux[idx] = U0 * sin(2.0 * pi * x / L) * cos(2.0 * pi * y / L);
                uy[idx] = -U0 * cos(2.0 * pi * x / L) * sin(2.0 * pi * y / L);
                uz[idx] = 0.0;
                double pp = -(U0 * U0 / 4.0) * (cos(4.0 * pi * x / L) + cos(4.0 * pi * y / L));
                rho[idx] = 1.0 + 3.0 * pp;
            }
    tg_fill(P, f, rho, ux, uy, uz);
}

/* second-order equilibrium start, Cavity/initial.f90:3-34 with
 * feq of Cavity/collision.f90:103-114 */
void orc_init_equilibrium2(const orc_params *P, double *f, const double *rho, const double *ux,
                           const double *uy, const double *uz) {
    const orc_lattice *L = &P->lat;
    const long N = (long)P->nx * P->ny * P->nz;
    for (long idx = 0; idx < N; idx++)
        for (int ip = 0; ip < L->q; ip++) {
            double u9 = ux[idx], v9 = uy[idx], w9 = uz[idx];
            double eu = (L->cx[ip] * u9 + L->cy[ip] * v9 + L->cz[ip] * w9) / L->rt;
            double uv = (u9 * u9 + v9 * v9 + w9 * w9) / L->rt;
            f[ip * N + idx] = L->w[ip] * rho[idx] * (1. + eu + 0.5 * (eu * eu - uv));
        }
}

/* channel start of init_arrays, initial.cu:268-326 (log-law mean flow with
 * the log10 of the reference, and f at rest minus the force shift) */
void orc_init_channel_loglaw(const orc_params *P, double ustar, double ystar, double *f,
                             double *rho, double *ux, double *uy, double *uz) {
    const orc_lattice *L = &P->lat;
    const int LX = P->nx, LY = P->ny, LZ = P->nz;
    const long N = (long)LX * LY * LZ;
    const double pi2 = 2 * acos(-1.0);
    for (int iz = 0; iz < LZ; iz++)
        for (int iy = 0; iy < LY; iy++)
            for (int ix = 0; ix < LX; ix++) {
                long idx = ((long)iz * LY + iy) * LX + ix;
                rho[idx] = 1.0;
                double A9 = 0.1 * sqrt(2.0), alpha = 1.0, beta9 = 1.0, cc = 60.0;
                double ccc1 = -LX / pi2 / alpha / ystar * A9 * ustar / cc / cc;
                uy[idx] = 0.0;
                uz[idx] = 0.0;
                double z9 = pi2 * (iz + 0.5) / LZ;
                double x9 = pi2 * (ix + 0.5) / LX;
                double yplus = iy <= LY / 2 ? (iy + 0.5) / ystar : (LY - iy - 0.5) / ystar;
                double u;
                if (yplus <= 10.8) {
                    u = ustar * yplus;
                } else {
                    u = log10(yplus) / 0.41 + 5.0;
                    u *= ustar;
                }
                double uu9 = ccc1 * yplus * sin(alpha * x9 + beta9 * z9);
                ux[idx] = u + uu9;
                double usq = 0.0;
                for (int ip = 0; ip < L->q; ip++) {
                    double feq = L->w[ip] * rho[idx] * (1.0 - 1.5 * usq);
                    f[ip * N + idx] = feq - 0.5 * P->force[0] * L->cx[ip] / (1.0 / 3.0) * feq;
                }
            }
}

/* counter-based generator: splitmix64 finaliser on (seed, node, component) */
uint64_t orc_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

double orc_uniform_pm1(uint64_t seed, uint64_t node, uint64_t comp) {
    uint64_t h = orc_splitmix64(seed ^ orc_splitmix64(node * 4u + comp));
    /* 53 random bits -> [0,1) -> [-1,1) */
    double r = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    return 2.0 * r - 1.0;
}

/* channel start of the 384x192x128 workload: laminar parabola with centreline
 * uc across the wall-normal (y) axis, walls half a cell outside the first and
 * last rows, plus amp*uc uniform noise on all three components; f is the
 * second-order equilibrium of that state. */
void orc_init_channel_config(const orc_params *P, double uc, double amp, uint64_t seed,
                             double *f, double *rho, double *ux, double *uy, double *uz) {
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const long N = (long)nx * ny * nz;
    const double H = ny;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                long idx = ((long)z * ny + y) * nx + x;
                double yy = y + 0.5;
                double up = 4.0 * uc * yy * (H - yy) / (H * H);
                rho[idx] = 1.0;
                ux[idx] = up + amp * uc * orc_uniform_pm1(seed, (uint64_t)idx, 0);
                uy[idx] = amp * uc * orc_uniform_pm1(seed, (uint64_t)idx, 1);
                uz[idx] = amp * uc * orc_uniform_pm1(seed, (uint64_t)idx, 2);
            }
    (void)N;
    orc_init_equilibrium2(P, f, rho, ux, uy, uz);
}


/* ---- the reference's file writers (output.cu) -------------------------- */

static FILE *orc_open(const char *dir, const char *name, const char *mode) {
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    return fopen(path, mode);
}

/* output.cu:24-56: sums in index order, then the console line and the
 * statistics.dat line */
int orc_out_diag(const char *dir, int istep, long n, const double *rho, const double *ux, const double *uy,
                 const double *uz, double u0) {
    double umean = 0.0, vmean = 0.0, wmean = 0.0, rhomean = 0.0;
    for (long i = 0; i < n; i++) {
        umean += ux[i];
        vmean += uy[i];
        wmean += uz[i];
        rhomean += rho[i];
    }
    umean /= n;
    vmean /= n;
    wmean /= n;
    rhomean /= n;
    printf("Step %-7d umean = %.17e, vmean = %.17e, wmean = %.17e, rhomean = %14.6e\n", istep, umean / u0, vmean,
           wmean, rhomean);
    fflush(stdout);
    FILE *fp = orc_open(dir, "statistics.dat", "a");
    if (!fp) return -1;
    const int w = fprintf(fp, "%-7d %14.6e %14.6e %14.6e %14.6e\n", istep, umean, vmean, wmean, rhomean);
    fclose(fp);
    return w < 0 ? -1 : 0;
}

/* output.cu:89-131: rho, ux, uy, uz back to back */
int orc_out_flow(const char *dir, int istep, long n, const double *rho, const double *ux, const double *uy,
                 const double *uz) {
    char name[64];
    snprintf(name, sizeof name, "%09d.dat", istep);
    FILE *fp = orc_open(dir, name, "wb");
    if (!fp) return -1;
    const double *a[4] = {rho, ux, uy, uz};
    int ok = 1;
    for (int k = 0; k < 4; k++) ok = ok && fwrite(a[k], sizeof(double), (size_t)n, fp) == (size_t)n;
    fclose(fp);
    return ok ? 0 : -1;
}

/* output.cu:158-214: per y plane, the means over x (outer) and z (inner),
 * then the second moments of the fluctuations in the same order */
int orc_out_profile(const char *dir, int istep, int nx, int ny, int nz, const double *ux, const double *uy,
                    const double *uz, const double *taut, double ystar) {
    FILE *fp = orc_open(dir, "Profiles.txt", "a");
    if (!fp) return -1;
    fprintf(fp, "%d\n", istep);
    for (int iy = 0; iy < ny; iy++) {
        double su = 0.0, sv = 0.0, sw = 0.0, st = 0.0;
        double s_uu = 0, s_vv = 0, s_ww = 0, s_uv = 0, s_uw = 0, s_vw = 0;
        int count = 0;
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const long idx = ((long)iz * ny + iy) * nx + ix;
                su += ux[idx];
                sv += uy[idx];
                sw += uz[idx];
                st += taut[idx];
                count++;
            }
        const double au = su / count, av = sv / count, aw = sw / count;
        (void)st;
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const long idx = ((long)iz * ny + iy) * nx + ix;
                const double ur = ux[idx] - au, vr = uy[idx] - av, wr = uz[idx] - aw;
                s_uu += ur * ur;
                s_vv += vr * vr;
                s_ww += wr * wr;
                s_uv += ur * vr;
                s_uw += ur * wr;
                s_vw += vr * wr;
            }
        fprintf(fp, "%d, %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e %14.6e\n", iy,
                iy + 0.5, (iy + 0.5) / ystar, au, av, aw, s_uu / count, s_vv / count, s_ww / count, s_uv / count,
                s_uw / count, s_vw / count);
    }
    const int e = fflush(fp);
    fclose(fp);
    return e == 0 ? 0 : -1;
}

/* output.cu:227-258: all populations, reference layout */
int orc_out_f(const char *dir, int istep, int q, long n, const double *f) {
    char name[64];
    snprintf(name, sizeof name, "f%09d.dat", istep);
    FILE *fp = orc_open(dir, name, "wb");
    if (!fp) return -1;
    const size_t cnt = (size_t)q * (size_t)n;
    const int ok = fwrite(f, sizeof(double), cnt, fp) == cnt;
    fclose(fp);
    return ok ? 0 : -1;
}
