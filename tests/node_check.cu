// node_check.cu -- host-side check of the solver's per-node arithmetic
// (recursively-regularized-lbm_gb300/csrc/rr_node.cuh, compiled for the CPU)
// against the oracle's restatement of the reference (oracle/rr_oracle.c).
// Built and run by tests/test_node_cpu.py; needs no GPU.
//
// For random post-stream states it compares, in FP64:
//   moments27 / collide27 / collide27_forced (factored D3Q27) with
//   moments_generic / collide_generic
//   collide (D3Q27 and D3Q19, with and without body force) with orc_collide_node
//   regularize (wall closure) with orc_regularize_node
// and the FP32 forms with the FP64 ones.  Prints the largest differences;
// exits 1 if one exceeds its bound.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "rr_node.cuh"

extern "C" {
#include "rr_oracle.h"
}

using namespace rr;

static int failures = 0;
static void check(const char *what, double err, double bound) {
    printf("%-44s max err %.3e (bound %.1e)%s\n", what, err, bound, err <= bound ? "" : "  FAIL");
    if (!(err <= bound)) failures++;
}

template <class LT>
static void random_state(std::mt19937_64 &g, double amp, double (&f)[LT::Q], double (&d)[LT::Q],
                         const orc_lattice &L) {
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    // a near-equilibrium state with a velocity and a non-equilibrium part
    double rho = 1.0 + 0.02 * U(g), u[3] = {amp * U(g), amp * U(g), amp * U(g)};
    for (int i = 0; i < LT::Q; i++) {
        double fe = orc_feq(&L, i, rho, u[0], u[1], u[2]);
        f[i] = fe * (1.0 + 0.01 * U(g));
        d[i] = f[i] / LT::w(i) - 1.0;
    }
}

template <class LT, bool FORCE>
static void run(const char *name, int order, double F0) {
    orc_lattice L;
    orc_lattice_init(&L, LT::Q, order, ORC_CS_SQRT_RT);
    std::mt19937_64 g(12345 + LT::Q + (FORCE ? 7 : 0));
    const double F[3] = {FORCE ? F0 : 0.0, FORCE ? -0.6 * F0 : 0.0, FORCE ? 0.3 * F0 : 0.0};
    double e_mom = 0, e_col = 0, e_reg = 0, e_fac = 0, e_f32 = 0;
    for (int trial = 0; trial < 2000; trial++) {
        double f[LT::Q], d[LT::Q];
        random_state<LT>(g, 0.1, f, d, L);
        // moments against the oracle's macrovar
        Mom<double> m = moments<LT>(d);
        double ux, uy, uz;
        velocity(m, F[0], F[1], F[2], ux, uy, uz);
        double r_o, u_o, v_o, w_o;
        orc_moments_node(&L, F, f, &r_o, &u_o, &v_o, &w_o);
        e_mom = fmax(e_mom, fabs(1.0 + m.drho - r_o));
        e_mom = fmax(e_mom, fmax(fabs(ux - u_o), fmax(fabs(uy - v_o), fabs(uz - w_o))));
        if constexpr (LT::Q == 27) {
            Mom<double> mg = moments_generic<LT>(d);
            const double *a = &m.drho, *b = &mg.drho;
            for (int k = 0; k < 10; k++) e_fac = fmax(e_fac, fabs(a[k] - b[k]));
        }
        // collision with a given tau
        const double tau = 0.52 + 0.4 * (trial % 7) / 7.0;
        double dc[LT::Q], fo[LT::Q];
        for (int i = 0; i < LT::Q; i++) {
            dc[i] = d[i];
            fo[i] = f[i];
        }
        collide<LT, double, FORCE>(dc, m, m.drho, ux, uy, uz, 1.0 - 1.0 / tau, F[0], F[1], F[2]);
        orc_collide_node(&L, tau, F, r_o, u_o, v_o, w_o, fo);
        for (int i = 0; i < LT::Q; i++) e_col = fmax(e_col, fabs(LT::w(i) * (1.0 + dc[i]) - fo[i]));
        if constexpr (LT::Q == 27) {
            // the factored D3Q27 forms (collide27, collide27_forced) against the pair loop
            double dg[LT::Q];
            for (int i = 0; i < LT::Q; i++) dg[i] = d[i];
            collide_generic<LT, double, FORCE>(dg, m, m.drho, ux, uy, uz, 1.0 - 1.0 / tau, F[0], F[1], F[2]);
            for (int i = 0; i < LT::Q; i++) e_fac = fmax(e_fac, fabs(dg[i] - dc[i]));
        }
        // FP32 path against FP64
        {
            float df[LT::Q];
            for (int i = 0; i < LT::Q; i++) df[i] = (float)d[i];
            Mom<float> mf = moments<LT>(df);
            float uxf, uyf, uzf;
            velocity(mf, (float)F[0], (float)F[1], (float)F[2], uxf, uyf, uzf);
            collide<LT, float, FORCE>(df, mf, mf.drho, uxf, uyf, uzf, (float)(1.0 - 1.0 / tau), (float)F[0],
                                      (float)F[1], (float)F[2]);
            for (int i = 0; i < LT::Q; i++) e_f32 = fmax(e_f32, fabs((double)df[i] - dc[i]));
        }
        // wall closure of the populations entering through the y-lo face
        int ent[27] = {0};
        uint32_t mask = 0;
        for (int i = 0; i < LT::Q; i++)
            if (LT::cy(i) > 0) {
                ent[i] = 1;
                mask |= 1u << i;
            }
        double dr[LT::Q], fr[LT::Q];
        for (int i = 0; i < LT::Q; i++) {
            dr[i] = d[i];
            fr[i] = f[i];
        }
        regularize<LT, double, FORCE>(dr, mask, F[0], F[1], F[2]);
        orc_regularize_node(&L, F, fr, ent);
        for (int i = 0; i < LT::Q; i++) e_reg = fmax(e_reg, fabs(LT::w(i) * (1.0 + dr[i]) - fr[i]));
    }
    char buf[128];
    snprintf(buf, sizeof buf, "%s moments vs oracle", name);
    check(buf, e_mom, 1e-15);
    snprintf(buf, sizeof buf, "%s collision vs oracle", name);
    check(buf, e_col, 1e-15);
    snprintf(buf, sizeof buf, "%s wall closure vs oracle", name);
    check(buf, e_reg, 1e-15);
    if (LT::Q == 27) {
        snprintf(buf, sizeof buf, "%s factored vs generic form", name);
        check(buf, e_fac, 1e-15);
    }
    snprintf(buf, sizeof buf, "%s FP32 vs FP64 deviations", name);
    check(buf, e_f32, 2e-6);
}

int main() {
    run<L27, false>("D3Q27", ORC_ORDER_CUDA, 0.0);
    run<L27, true>("D3Q27 + force", ORC_ORDER_CUDA, 1e-4);
    run<L19, false>("D3Q19", ORC_ORDER_FORTRAN, 0.0);
    run<L19, true>("D3Q19 + force", ORC_ORDER_FORTRAN, 1e-4);
    printf(failures ? "FAILED\n" : "OK\n");
    return failures ? 1 : 0;
}
