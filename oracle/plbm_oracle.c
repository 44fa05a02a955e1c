/*
 * plbm_oracle.c -- CPU restatement of the periodic-lbm D2Q9 hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product links, loads or calls this file.
 *
 * Parity status: pinned to the reference binary's printed Taylor-Green errors
 * for the finite-difference Bardow streaming with BGK (graphs/fvm_bardow_64.txt;
 * tests/test_reference_bardow64.py); unpinned for TRT, RR, the improved BGK and
 * lbm_stream (no Fortran compiler on either machine; the reference holds no
 * other output for them).  See plbm_oracle.h.  Each
 * routine cites the Fortran it restates and keeps the Fortran evaluation
 * order: Fortran evaluates a+b+c as (a+b)+c and a*b*c as (a*b)*c and never
 * breaks parentheses, so every expression below is written with the same
 * association.  Built with -ffp-contract=off for the strict oracle, so that
 * each + - * / is one IEEE-754 binary64 operation, exactly as gfortran emits
 * it without FMA contraction.
 *
 * Index conventions are in plbm_oracle.h.  Loops keep the reference order
 * (x outer, y inner) and its OpenMP worksharing; the per-cell arithmetic does
 * not depend on the thread count.
 */
#include "plbm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(y, x, q) ((size_t)(y) + (size_t)ld * ((size_t)(x) + (size_t)nx * (size_t)(q)))

/* D2Q9 weights, src/fvm_bardow.F90:90-92 */
static const double W0 = 4.0 / 9.0, WS = 1.0 / 9.0, WD = 1.0 / 36.0;
static const double CSQR = 1.0 / 3.0;

int oref_pad16(int ny)
{
    /* src/fvm_bardow.F90:144-147 */
    int rmd = ny % 16;
    return rmd > 0 ? ny + (16 - rmd) : ny;
}

int oref_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Fortran mod(a,n)+1 wrap maps, 1-based (src/periodic_lbm.f90:63-64,79-80). */
static inline int xp1_of(int x1, int n) { return (x1 % n) + 1; }
static inline int xm1_of(int x1, int n) { return ((n + x1 - 2) % n) + 1; }

/* ------------------------------------------------------------------------ */
/* src/periodic_lbm.f90:45-127                                               */
void oref_lbm_stream(int nx, int ny, int ld, const double *fsrc, double *fdst)
{
    /* :57  fdst(1:ny,:,0) = fsrc(1:ny,:,0) */
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++)
            fdst[IDX(y, x, 0)] = fsrc[IDX(y, x, 0)];
    /* :60-71 */
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        int xp1 = xp1_of(x1, nx), xm1 = xm1_of(x1, nx);
        for (int y1 = 1; y1 <= ny; y1++) {
            fdst[IDX(y1 - 1, x1 - 1, 1)] = fsrc[IDX(y1 - 1, xm1 - 1, 1)];
            fdst[IDX(y1 - 1, x1 - 1, 3)] = fsrc[IDX(y1 - 1, xp1 - 1, 3)];
        }
    }
    /* :74-86 */
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        for (int y1 = 1; y1 <= ny; y1++) {
            int yp1 = xp1_of(y1, ny), ym1 = xm1_of(y1, ny);
            fdst[IDX(y1 - 1, x1 - 1, 2)] = fsrc[IDX(ym1 - 1, x1 - 1, 2)];
            fdst[IDX(y1 - 1, x1 - 1, 4)] = fsrc[IDX(yp1 - 1, x1 - 1, 4)];
        }
    }
    /* :89-105 */
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        int xp1 = xp1_of(x1, nx), xm1 = xm1_of(x1, nx);
        for (int y1 = 1; y1 <= ny; y1++) {
            int yp1 = xp1_of(y1, ny), ym1 = xm1_of(y1, ny);
            fdst[IDX(y1 - 1, x1 - 1, 5)] = fsrc[IDX(ym1 - 1, xm1 - 1, 5)];
            fdst[IDX(y1 - 1, x1 - 1, 7)] = fsrc[IDX(yp1 - 1, xp1 - 1, 7)];
        }
    }
    /* :107-123 */
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        int xp1 = xp1_of(x1, nx), xm1 = xm1_of(x1, nx);
        for (int y1 = 1; y1 <= ny; y1++) {
            int yp1 = xp1_of(y1, ny), ym1 = xm1_of(y1, ny);
            fdst[IDX(y1 - 1, x1 - 1, 6)] = fsrc[IDX(ym1 - 1, xp1 - 1, 6)];
            fdst[IDX(y1 - 1, x1 - 1, 8)] = fsrc[IDX(yp1 - 1, xm1 - 1, 8)];
        }
    }
}

/* ------------------------------------------------------------------------ */
/* src/fvm_bardow.F90:99-126                                                 */
void oref_equilibrium(double rho, double ux, double uy, double feq[9])
{
    double uxx = ux * ux;
    double uyy = uy * uy;
    double indp = 1.0 - 1.5 * (uxx + uyy);
    feq[0] = W0 * rho * (indp);
    feq[1] = WS * rho * (indp + 3.0 * ux + 4.5 * uxx);
    feq[2] = WS * rho * (indp + 3.0 * uy + 4.5 * uyy);
    feq[3] = WS * rho * (indp - 3.0 * ux + 4.5 * uxx);
    feq[4] = WS * rho * (indp - 3.0 * uy + 4.5 * uyy);
    double uxpy = ux + uy;
    feq[5] = WD * rho * (indp + 3.0 * uxpy + 4.5 * uxpy * uxpy);
    feq[7] = WD * rho * (indp - 3.0 * uxpy + 4.5 * uxpy * uxpy);
    double uxmy = ux - uy;
    feq[6] = WD * rho * (indp - 3.0 * uxmy + 4.5 * uxmy * uxmy);
    feq[8] = WD * rho * (indp + 3.0 * uxmy + 4.5 * uxmy * uxmy);
}

/* ------------------------------------------------------------------------ */
/* src/collision_bgk.F90:35-82 (bgk_kernel) and :84-176 (bgk_kernel_cache)   */
void oref_collide_bgk(int nx, int ny, int ld, double *f, double omega, int split)
{
    if (!split) {
        double omegabar = 1.0 - omega;
#pragma omp parallel for schedule(static)
        for (int x = 0; x < nx; x++) {
            for (int y = 0; y < ny; y++) {
                double fs[9], feq[9];
                for (int q = 0; q < 9; q++) fs[q] = f[IDX(y, x, q)];
                double rho = (((fs[5] + fs[7]) + (fs[6] + fs[8])) +
                              ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
                double invrho = 1.0 / rho;
                double ux = invrho * (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3]));
                double uy = invrho * (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4]));
                oref_equilibrium(rho, ux, uy, feq);
                for (int q = 0; q < 9; q++) f[IDX(y, x, q)] = omegabar * fs[q] + omega * feq[q];
            }
        }
        return;
    }
    /* split variant: bgk_kernel_cache */
    const double one_third = 1.0 / 3.0;
    double omegabar = 1.0 - omega;
    double omega_w0 = 3.0 * omega * W0;
    double omega_ws = 3.0 * omega * WS;
    double omega_wd = 3.0 * omega * WD;
#pragma omp parallel
    {
        double *rho = malloc(sizeof(double) * (size_t)ny);
        double *ux = malloc(sizeof(double) * (size_t)ny);
        double *uy = malloc(sizeof(double) * (size_t)ny);
        double *indp = malloc(sizeof(double) * (size_t)ny);
#pragma omp for schedule(static)
        for (int x = 0; x < nx; x++) {
            for (int y = 0; y < ny; y++) {
                double fs[9];
                for (int q = 0; q < 9; q++) fs[q] = f[IDX(y, x, q)];
                rho[y] = (((fs[5] + fs[7]) + (fs[6] + fs[8])) +
                          ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
                double invrho = 1.0 / rho[y];
                ux[y] = invrho * (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3]));
                uy[y] = invrho * (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4]));
                indp[y] = one_third - 0.5 * (ux[y] * ux[y] + uy[y] * uy[y]);
                f[IDX(y, x, 0)] = omegabar * fs[0] + omega_w0 * rho[y] * indp[y];
            }
            for (int y = 0; y < ny; y++) {
                double v = indp[y] + 1.5 * ux[y] * ux[y];
                f[IDX(y, x, 1)] = omegabar * f[IDX(y, x, 1)] + omega_ws * rho[y] * (v + ux[y]);
                f[IDX(y, x, 3)] = omegabar * f[IDX(y, x, 3)] + omega_ws * rho[y] * (v - ux[y]);
            }
            for (int y = 0; y < ny; y++) {
                double v = indp[y] + 1.5 * uy[y] * uy[y];
                f[IDX(y, x, 2)] = omegabar * f[IDX(y, x, 2)] + omega_ws * rho[y] * (v + uy[y]);
                f[IDX(y, x, 4)] = omegabar * f[IDX(y, x, 4)] + omega_ws * rho[y] * (v - uy[y]);
            }
            for (int y = 0; y < ny; y++) {
                double velxpy = ux[y] + uy[y];
                double v = indp[y] + 1.5 * velxpy * velxpy;
                f[IDX(y, x, 5)] = omegabar * f[IDX(y, x, 5)] + omega_wd * rho[y] * (v + velxpy);
                f[IDX(y, x, 7)] = omegabar * f[IDX(y, x, 7)] + omega_wd * rho[y] * (v - velxpy);
            }
            for (int y = 0; y < ny; y++) {
                double velxmy = ux[y] - uy[y];
                double v = indp[y] + 1.5 * velxmy * velxmy;
                f[IDX(y, x, 6)] = omegabar * f[IDX(y, x, 6)] + omega_wd * rho[y] * (v - velxmy);
                f[IDX(y, x, 8)] = omegabar * f[IDX(y, x, 8)] + omega_wd * rho[y] * (v + velxmy);
            }
        }
        free(rho); free(ux); free(uy); free(indp);
    }
}

/* ------------------------------------------------------------------------ */
/* src/collision_trt.F90:24-34                                               */
double oref_magic_number(double le, double ld)
{
    return (2.0 - le) * (2.0 - ld) / (4.0 * le * ld);
}

double oref_lambda_d(double omega, double x)
{
    return (4.0 - 2.0 * omega) / (4.0 * x * omega + 2.0 - omega);
}

/* src/collision_trt.F90:12-20 */
static const double T0 = 4.0 / 9.0;
static const double T1X2 = (1.0 / 9.0) * 2.0;
static const double T2X2 = (1.0 / 36.0) * 2.0;
static const double INV2CSQ2 = 1.0 / (2.0 * (1.0 / 3.0) * (1.0 / 3.0));
#define FAC1 (T1X2 * INV2CSQ2)
#define FAC2 (T2X2 * INV2CSQ2)

/* src/collision_trt.F90:64-160 (trt_naive) and :162-290 (trt_split) */
void oref_collide_trt(int nx, int ny, int ld, double *f, double lambda_e, double lambda_d, int split)
{
    const double fac1 = FAC1, fac2 = FAC2;
    double les = 0.5 * lambda_e;
    double lds = 0.5 * lambda_d;
    if (!split) {
#pragma omp parallel for schedule(static)
        for (int x = 0; x < nx; x++) {
            for (int y = 0; y < ny; y++) {
                double vC = f[IDX(y, x, 0)], vE = f[IDX(y, x, 1)], vN = f[IDX(y, x, 2)];
                double vW = f[IDX(y, x, 3)], vS = f[IDX(y, x, 4)], vNE = f[IDX(y, x, 5)];
                double vNW = f[IDX(y, x, 6)], vSW = f[IDX(y, x, 7)], vSE = f[IDX(y, x, 8)];
                double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
                double velX = (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
                double velY = (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
                double velX2 = velX * velX;
                double velY2 = velY * velY;
                double feq_common = rho - 1.5 * (velX2 + velY2);
                f[IDX(y, x, 0)] = vC * (1.0 - lambda_e) + lambda_e * T0 * feq_common;
                double velXPY = velX + velY;
                double sym = les * (vNE + vSW - fac2 * velXPY * velXPY - T2X2 * feq_common);
                double asym = lds * (vNE - vSW - 3.0 * T2X2 * velXPY);
                f[IDX(y, x, 5)] = vNE - sym - asym;
                f[IDX(y, x, 7)] = vSW - sym + asym;
                double velXMY = velX - velY;
                sym = les * (vSE + vNW - fac2 * velXMY * velXMY - T2X2 * feq_common);
                asym = lds * (vSE - vNW - 3.0 * T2X2 * velXMY);
                f[IDX(y, x, 8)] = vSE - sym - asym;
                f[IDX(y, x, 6)] = vNW - sym + asym;
                sym = les * (vN + vS - fac1 * velY2 - T1X2 * feq_common);
                asym = lds * (vN - vS - 3.0 * T1X2 * velY);
                f[IDX(y, x, 2)] = vN - sym - asym;
                f[IDX(y, x, 4)] = vS - sym + asym;
                sym = les * (vE + vW - fac1 * velX2 - T1X2 * feq_common);
                asym = lds * (vE - vW - 3.0 * T1X2 * velX);
                f[IDX(y, x, 1)] = vE - sym - asym;
                f[IDX(y, x, 3)] = vW - sym + asym;
            }
        }
        return;
    }
#pragma omp parallel
    {
        double *rho = malloc(sizeof(double) * (size_t)ny);
        double *velX = malloc(sizeof(double) * (size_t)ny);
        double *velY = malloc(sizeof(double) * (size_t)ny);
        double *fc = malloc(sizeof(double) * (size_t)ny);
#pragma omp for schedule(static)
        for (int x = 0; x < nx; x++) {
            for (int y = 0; y < ny; y++) {
                double vC = f[IDX(y, x, 0)], vE = f[IDX(y, x, 1)], vN = f[IDX(y, x, 2)];
                double vW = f[IDX(y, x, 3)], vS = f[IDX(y, x, 4)], vNE = f[IDX(y, x, 5)];
                double vNW = f[IDX(y, x, 6)], vSW = f[IDX(y, x, 7)], vSE = f[IDX(y, x, 8)];
                rho[y] = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
                velX[y] = (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
                velY[y] = (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
                fc[y] = rho[y] - 1.5 * (velX[y] * velX[y] + velY[y] * velY[y]);
                f[IDX(y, x, 0)] = vC * (1.0 - lambda_e) + lambda_e * T0 * fc[y];
            }
            for (int y = 0; y < ny; y++) {
                double vNE = f[IDX(y, x, 5)], vSW = f[IDX(y, x, 7)];
                double velXPY = velX[y] + velY[y];
                double sym = les * (vNE + vSW - fac2 * velXPY * velXPY - T2X2 * fc[y]);
                double asym = lds * (vNE - vSW - 3.0 * T2X2 * velXPY);
                f[IDX(y, x, 5)] = f[IDX(y, x, 5)] - sym - asym;
                f[IDX(y, x, 7)] = f[IDX(y, x, 7)] - sym + asym;
            }
            for (int y = 0; y < ny; y++) {
                double vNW = f[IDX(y, x, 6)], vSE = f[IDX(y, x, 8)];
                double velXMY = velX[y] - velY[y];
                double sym = les * (vSE + vNW - fac2 * velXMY * velXMY - T2X2 * fc[y]);
                double asym = lds * (vSE - vNW - 3.0 * T2X2 * velXMY);
                f[IDX(y, x, 8)] = f[IDX(y, x, 8)] - sym - asym;
                f[IDX(y, x, 6)] = f[IDX(y, x, 6)] - sym + asym;
            }
            for (int y = 0; y < ny; y++) {
                double vN = f[IDX(y, x, 2)], vS = f[IDX(y, x, 4)];
                double sym = les * (vN + vS - fac1 * velY[y] * velY[y] - T1X2 * fc[y]);
                double asym = lds * (vN - vS - 3.0 * T1X2 * velY[y]);
                f[IDX(y, x, 2)] = f[IDX(y, x, 2)] - sym - asym;
                f[IDX(y, x, 4)] = f[IDX(y, x, 4)] - sym + asym;
            }
            for (int y = 0; y < ny; y++) {
                double vE = f[IDX(y, x, 1)], vW = f[IDX(y, x, 3)];
                double sym = les * (vE + vW - fac1 * velX[y] * velX[y] - T1X2 * fc[y]);
                double asym = lds * (vE - vW - 3.0 * T1X2 * velX[y]);
                f[IDX(y, x, 1)] = f[IDX(y, x, 1)] - sym - asym;
                f[IDX(y, x, 3)] = f[IDX(y, x, 3)] - sym + asym;
            }
        }
        free(rho); free(velX); free(velY); free(fc);
    }
}

/* ------------------------------------------------------------------------ */
/* src/collision_regularized.F90:40-202 (rr_kernel_naive)                    */
void oref_collide_rr(int nx, int ny, int ld, double *f, double omega)
{
    double omega_w0 = W0 * (1.0 - omega);
    double omega_ws = WS * (1.0 - omega);
    double omega_wd = WD * (1.0 - omega);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; x++) {
        for (int y = 0; y < ny; y++) {
            double feq[9];
            double vC = f[IDX(y, x, 0)], vE = f[IDX(y, x, 1)], vN = f[IDX(y, x, 2)];
            double vW = f[IDX(y, x, 3)], vS = f[IDX(y, x, 4)], vNE = f[IDX(y, x, 5)];
            double vNW = f[IDX(y, x, 6)], vSW = f[IDX(y, x, 7)], vSE = f[IDX(y, x, 8)];
            double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
            double invrho = 1.0 / rho;
            double ux = invrho * (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
            double uy = invrho * (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
            double uxx = ux * ux;
            double uyy = uy * uy;
            double uxxy = uxx * uy;
            double uyyx = uyy * ux;
            double uxxyy = uxx * uyy;
            double indp0 = 1.0 - 1.5 * (uxx + uyy);
            double indps = indp0 - 4.5 * uxxyy;
            double indpd = indp0 + 9.0 * uxxyy;
            indp0 = indp0 + 2.25 * uxxyy;
            feq[0] = W0 * rho * indp0;
            feq[1] = WS * rho * (indps + 3.0 * ux + 4.5 * (uxx - uyyx));
            feq[3] = WS * rho * (indps - 3.0 * ux + 4.5 * (uxx + uyyx));
            feq[2] = WS * rho * (indps + 3.0 * uy + 4.5 * (uyy - uxxy));
            feq[4] = WS * rho * (indps - 3.0 * uy + 4.5 * (uyy + uxxy));
            vC = vC - feq[0];
            vE = vE - feq[1];
            vN = vN - feq[2];
            vW = vW - feq[3];
            vS = vS - feq[4];
            double axx = CSQR * (2.0 * (vE + vW) - (vN + vS) - vC);
            double ayy = CSQR * (2.0 * (vN + vS) - (vE + vW) - vC);
            double u3p = uxxy + uyyx;
            double uxpy = ux + uy;
            double indp57 = indpd + 4.5 * uxpy * uxpy;
            feq[5] = WD * rho * (indp57 + 3.0 * uxpy + 9.0 * u3p);
            feq[7] = WD * rho * (indp57 - 3.0 * uxpy - 9.0 * u3p);
            double u3m = uxxy - uyyx;
            double uxmy = ux - uy;
            double indp68 = indpd + 4.5 * uxmy * uxmy;
            feq[6] = WD * rho * (indp68 - 3.0 * uxmy + 9.0 * u3m);
            feq[8] = WD * rho * (indp68 + 3.0 * uxmy - 9.0 * u3m);
            vNE = vNE - feq[5];
            vNW = vNW - feq[6];
            vSW = vSW - feq[7];
            vSE = vSE - feq[8];
            double tmp = 2.0 * CSQR * (vNE + vNW + vSW + vSE);
            axx = axx + tmp;
            ayy = ayy + tmp;
            double axy = ((vNE + vSW) - (vNW + vSE));
            double axxy = 2.0 * ux * axy + uy * axx;
            double ayyx = 2.0 * uy * axy + ux * ayy;
            double axxyy = 2.0 * (ux * ayyx + uy * axxy) - uxx * ayy - uyy * axx - 4.0 * ux * uy * axy;
            indp0 = -1.5 * (axx + ayy);
            indps = indp0 - 4.5 * axxyy;
            indpd = 9.0 * axxyy - 2.0 * indp0;
            indp0 = indp0 + 2.25 * axxyy;
            vC = indp0;
            vE = indps + 4.5 * (axx - ayyx);
            vW = indps + 4.5 * (axx + ayyx);
            vN = indps + 4.5 * (ayy - axxy);
            vS = indps + 4.5 * (ayy + axxy);
            vNE = indpd + 9.0 * (axxy + ayyx + axy);
            vSW = indpd - 9.0 * (axxy + ayyx - axy);
            vNW = indpd + 9.0 * (axxy - ayyx - axy);
            vSE = indpd - 9.0 * (axxy - ayyx + axy);
            f[IDX(y, x, 0)] = feq[0] + omega_w0 * vC;
            f[IDX(y, x, 1)] = feq[1] + omega_ws * vE;
            f[IDX(y, x, 2)] = feq[2] + omega_ws * vN;
            f[IDX(y, x, 3)] = feq[3] + omega_ws * vW;
            f[IDX(y, x, 4)] = feq[4] + omega_ws * vS;
            f[IDX(y, x, 5)] = feq[5] + omega_wd * vNE;
            f[IDX(y, x, 6)] = feq[6] + omega_wd * vNW;
            f[IDX(y, x, 7)] = feq[7] + omega_wd * vSW;
            f[IDX(y, x, 8)] = feq[8] + omega_wd * vSE;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* src/collision_bgk_improved.f90:24-107.  The dummy is f1(ny,nx,0:8), so the */
/* buffer is addressed with row stride ny and plane stride ny*nx whatever ld */
/* the caller allocated (sequence association).                              */
void oref_collide_bgk_improved(int nx, int ny, double *f, double omega)
{
    const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
    double fac = 4.5 - 2.25 * omega;
    double omegabar = 1.0 - omega;
    size_t pl = (size_t)ny * (size_t)nx;
    for (int y = 0; y < ny; y++) {
        for (int x = 0; x < nx; x++) {
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            double vC = f[o], vE = f[o + pl], vN = f[o + 2 * pl], vW = f[o + 3 * pl];
            double vS = f[o + 4 * pl], vNE = f[o + 5 * pl], vNW = f[o + 6 * pl];
            double vSW = f[o + 7 * pl], vSE = f[o + 8 * pl];
            double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
            double invrho = 1.0 / rho;
            double sumX1 = vE + vNE + vSE;
            double sumXN = vW + vNW + vSW;
            double sumY1 = vN + vNE + vNW;
            double sumYN = vS + vSE + vSW;
            double m10 = invrho * (sumX1 - sumXN);
            double m01 = invrho * (sumY1 - sumYN);
            double u2 = m10 * m10;
            double v2 = m01 * m01;
            double m20 = invrho * (sumX1 + sumXN);
            double m02 = invrho * (sumY1 + sumYN);
            double Gx = fac * u2 * (m20 - one_third - u2);
            double Gy = fac * v2 * (m02 - one_third - v2);
            double X0 = -two_thirds + u2 + Gx;
            double X1 = -(X0 + 1.0 + m10) * 0.5;
            double XN = X1 + m10;
            double Y0 = -two_thirds + v2 + Gy;
            double Y1 = -(Y0 + 1.0 + m01) * 0.5;
            double YN = Y1 + m01;
            double rho_omega = rho * omega;
            X0 = X0 * rho_omega;
            X1 = X1 * rho_omega;
            XN = XN * rho_omega;
            f[o] = omegabar * vC + X0 * Y0;
            f[o + pl] = omegabar * vE + X1 * Y0;
            f[o + 2 * pl] = omegabar * vN + X0 * Y1;
            f[o + 3 * pl] = omegabar * vW + XN * Y0;
            f[o + 4 * pl] = omegabar * vS + X0 * YN;
            f[o + 5 * pl] = omegabar * vNE + X1 * Y1;
            f[o + 6 * pl] = omegabar * vNW + XN * Y1;
            f[o + 7 * pl] = omegabar * vSW + XN * YN;
            f[o + 8 * pl] = omegabar * vSE + X1 * YN;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* src/fvm_bardow.F90:356-388                                                */
void oref_update_macros(int nx, int ny, int ld, const double *f, double *grho, double *gux, double *guy)
{
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; x++) {
        for (int y = 0; y < ny; y++) {
            double fs[9];
            for (int q = 0; q < 9; q++) fs[q] = f[IDX(y, x, q)];
            double rho = fs[0] + (((fs[5] + fs[7]) + (fs[6] + fs[8])) +
                                  ((fs[1] + fs[3]) + (fs[2] + fs[4])));
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            grho[o] = rho;
            double invrho = 1.0 / rho;
            gux[o] = invrho * (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3]));
            guy[o] = invrho * (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4]));
        }
    }
}

/* ------------------------------------------------------------------------ */
/* src/vorticity.f90:13-43                                                   */
void oref_vorticity_2nd(int nx, int ny, const double *ux, const double *uy, double *w)
{
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        int xp1 = xp1_of(x1, nx), xm1 = xm1_of(x1, nx);
        for (int y1 = 1; y1 <= ny; y1++) {
            int yp1 = xp1_of(y1, ny), ym1 = xm1_of(y1, ny);
#define A2(a, yy, xx) a[(size_t)((yy) - 1) + (size_t)ny * (size_t)((xx) - 1)]
            double duydx = 0.5 * (A2(uy, y1, xp1) - A2(uy, y1, xm1));
            double duxdy = 0.5 * (A2(ux, yp1, x1) - A2(ux, ym1, x1));
            A2(w, y1, x1) = duydx - duxdy;
        }
    }
}

/* src/vorticity.f90:46-87 (t1 = 1/12 on the +-1 pair, t2 = 2/3 on the +-2 pair) */
void oref_vorticity_4th(int nx, int ny, const double *ux, const double *uy, double *w)
{
    const double t1 = 1.0 / 12.0, t2 = 2.0 / 3.0;
#pragma omp parallel for schedule(static)
    for (int x1 = 1; x1 <= nx; x1++) {
        int xp1 = (x1 % nx) + 1, xm1 = ((nx + x1 - 2) % nx) + 1;
        int xp2 = ((x1 + 1) % nx) + 1, xm2 = ((nx + x1 - 3) % nx) + 1;
        for (int y1 = 1; y1 <= ny; y1++) {
            int yp1 = (y1 % ny) + 1, ym1 = ((ny + y1 - 2) % ny) + 1;
            int yp2 = ((y1 + 1) % ny) + 1, ym2 = ((ny + y1 - 3) % ny) + 1;
            double duydx = t1 * (A2(uy, y1, xp1) - A2(uy, y1, xm1)) + t2 * (A2(uy, y1, xm2) - A2(uy, y1, xp2));
            double duxdy = t1 * (A2(ux, yp1, x1) - A2(ux, ym1, x1)) + t2 * (A2(ux, ym2, x1) - A2(ux, yp2, x1));
            A2(w, y1, x1) = duydx - duxdy;
        }
    }
}
#undef A2

/* ------------------------------------------------------------------------ */
/* src/fvm_bardow.F90:242-269                                                */
void oref_set_properties(double nu, double dt, const double *magic,
                         double *tau, double *omega, double *trt_magic)
{
    const double invcsqr = 1.0 / CSQR;
    double t = invcsqr * nu;
    *tau = t;
    *omega = dt / (t + 0.5 * dt);
    if (magic) *trt_magic = *magic;
    else {
        double r = t / dt;
        *trt_magic = r * r; /* (tau/dt)**2 */
    }
}

/* src/fvm_bardow.F90:272-305 */
void oref_set_pdf_to_equilibrium(int nx, int ny, int ld, const double *rho,
                                 const double *ux, const double *uy, double *f)
{
    for (int x = 0; x < nx; x++) {
        for (int y = 0; y < ny; y++) {
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            double feq[9];
            oref_equilibrium(rho[o], ux[o], uy[o], feq);
            for (int q = 0; q < 9; q++) f[IDX(y, x, q)] = feq[q];
        }
    }
}

/* src/periodic_lbm.f90:15-29 */
void oref_perform_lbm_step(int nx, int ny, int ld, double *f, int *iold, int *inew,
                           int kind, double omega, double trt_magic, int nsteps)
{
    size_t lat = (size_t)ld * (size_t)nx * 9u;
    for (int s = 0; s < nsteps; s++) {
        double *fo = f + (size_t)(*iold - 1) * lat;
        double *fn = f + (size_t)(*inew - 1) * lat;
        oref_lbm_stream(nx, ny, ld, fo, fn);
        switch (kind) {
        case OREF_BGK: oref_collide_bgk(nx, ny, ld, fn, omega, 0); break;
        case OREF_TRT: oref_collide_trt(nx, ny, ld, fn, omega, oref_lambda_d(omega, trt_magic), 0); break;
        case OREF_RR: oref_collide_rr(nx, ny, ld, fn, omega); break;
        case OREF_BGKI: oref_collide_bgk_improved(nx, ny, fn, omega); break;
        default: break;
        }
        int t = *iold;
        *iold = *inew;
        *inew = t;
    }
}

/* ------------------------------------------------------------------------ */
/* Finite-volume / finite-difference streaming (src/fvm_bardow.F90:393-886).  */
/* The reference loops x = 1, ny and y = 1, nx in stream_fvm_bardow and      */
/* stream_fdm_sofonea (:436,444 and :724,727...), which covers the grid only */
/* when nx == ny; these restatements loop over the whole grid (x = 1, nx,    */
/* y = 1, ny), identical for square grids.                                   */
static const double CXD[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const double CYD[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

/* stream_fvm_bardow, src/fvm_bardow.F90:409-506 (bilinear face values) */
void oref_stream_fvm_bardow(int nx, int ny, int ld, const double *fold, double *fnew, double dt)
{
    const double p2 = 0.5, p8 = 0.125;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) fnew[IDX(y, x, 0)] = fold[IDX(y, x, 0)];
    for (int q = 1; q <= 8; q++) {
        const double cxq = dt * CXD[q], cyq = dt * CYD[q];
#pragma omp parallel for schedule(static)
        for (int x1 = 1; x1 <= nx; x1++) {
            const int xp = xp1_of(x1, nx) - 1, xm = xm1_of(x1, nx) - 1, x = x1 - 1;
            for (int y1 = 1; y1 <= ny; y1++) {
                const int yp = xp1_of(y1, ny) - 1, ym = xm1_of(y1, ny) - 1, y = y1 - 1;
                const double fc = fold[IDX(y, x, q)], fe = fold[IDX(y, xp, q)], fn = fold[IDX(yp, x, q)];
                const double fw = fold[IDX(y, xm, q)], fs = fold[IDX(ym, x, q)];
                const double fne = fold[IDX(yp, xp, q)], fnw = fold[IDX(yp, xm, q)];
                const double fsw = fold[IDX(ym, xm, q)], fse = fold[IDX(ym, xp, q)];
                const double cfw = p2 * (fc + fw) - p2 * cxq * (fc - fw) - p8 * cyq * (fnw + fn - fsw - fs);
                const double cfn = p2 * (fc + fn) - p2 * cyq * (fn - fc) - p8 * cxq * (fne + fe - fnw - fw);
                const double cfe = p2 * (fc + fe) - p2 * cxq * (fe - fc) - p8 * cyq * (fne + fn - fse - fs);
                const double cfs = p2 * (fc + fs) - p2 * cyq * (fc - fs) - p8 * cxq * (fse + fe - fsw - fw);
                fnew[IDX(y, x, q)] = fc - cxq * (cfe - cfw) - cyq * (cfn - cfs);
            }
        }
    }
}

/* stream_fdm_bardow, src/fvm_bardow.F90:526-685.  variant 0: central
 * differences (the default build, :656-663); 1: isotropic differences of
 * Kumar 2004 (FDM_ISO, :645-655); 2: unweighted least squares (FDM_WLS,
 * :597-607); 3, 4: Gaussian-weighted least squares (FDM_WLS_GAUSS_V1 :604-624,
 * FDM_WLS_GAUSS_V2 :625-644, the reference's binary64 weights). */
void oref_stream_fdm_bardow(int nx, int ny, int ld, const double *fold, double *fnew, double dt, int variant)
{
    const double p2 = 0.5;
    const double two_thirds = 2.0 / 3.0, one_sixth = 1.0 / 6.0;
    const double five_sixths = 10.0 / 12.0, one_twelth = 1.0 / 12.0, one_third = 1.0 / 3.0;
    /* :561 fnew(:,:,0) = fold(:,:,0) (all ld rows) */
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ld; y++) fnew[IDX(y, x, 0)] = fold[IDX(y, x, 0)];
    for (int q = 1; q <= 8; q++) {
        const double cxq = dt * CXD[q], cyq = dt * CYD[q];
        const double cxxq = 0.5 * cxq * cxq, cyyq = 0.5 * cyq * cyq, cxyq = cxq * cyq;
#pragma omp parallel for schedule(static)
        for (int x1 = 1; x1 <= nx; x1++) {
            const int xp = xp1_of(x1, nx) - 1, xm = xm1_of(x1, nx) - 1, x = x1 - 1;
            for (int y1 = 1; y1 <= ny; y1++) {
                const int yp = xp1_of(y1, ny) - 1, ym = xm1_of(y1, ny) - 1, y = y1 - 1;
                const double fc = fold[IDX(y, x, q)], fe = fold[IDX(y, xp, q)], fn = fold[IDX(yp, x, q)];
                const double fw = fold[IDX(y, xm, q)], fs = fold[IDX(ym, x, q)];
                const double fne = fold[IDX(yp, xp, q)], fnw = fold[IDX(yp, xm, q)];
                const double fsw = fold[IDX(ym, xm, q)], fse = fold[IDX(ym, xp, q)];
                double dfx, dfy, dfxx, dfyy, dfxy;
                if (variant == 1) {
                    dfx = p2 * (one_sixth * (fne - fnw) + two_thirds * (fe - fw) + one_sixth * (fse - fsw));
                    dfy = p2 * (one_sixth * (fne - fse) + two_thirds * (fn - fs) + one_sixth * (fnw - fsw));
                    dfxx = one_twelth * (fne - 2 * fn + fnw) + five_sixths * (fe - 2 * fc + fw) +
                           one_twelth * (fse - 2 * fs + fsw);
                    dfyy = one_twelth * (fne - 2 * fe + fse) + five_sixths * (fn - 2 * fc + fs) +
                           one_twelth * (fnw - 2 * fw + fsw);
                    dfxy = 0.25 * (fne - fse - fnw + fsw);
                } else if (variant == 2) {
                    dfx = one_sixth * ((fne - fnw) + (fe - fw) + (fse - fsw));
                    dfy = one_sixth * ((fne - fse) + (fn - fs) + (fnw - fsw));
                    dfxx = one_third * (fne - 2 * fn + fnw) + one_third * (fe - 2 * fc + fw) +
                           one_third * (fse - 2 * fs + fsw);
                    dfyy = one_third * (fne - 2 * fe + fse) + one_third * (fn - 2 * fc + fs) +
                           one_third * (fnw - 2 * fw + fsw);
                    dfxy = 0.25 * (fne - fnw + fsw - fse);
                } else if (variant == 3 || variant == 4) {
                    const int g1 = variant == 3;
                    const double p1s = g1 ? 0.2880584423829145035434 : 0.3934930210807994210853;
                    const double p1d = g1 ? 0.1059707788085427065949 : 0.05325348945960039354075;
                    const double p2c = g1 ? -1.152233769531658458263 : -1.573972084323197018207;
                    const double p2d1 = g1 ? 0.5761168847658292291314 : 0.7869860421615988421706;
                    const double p2d2 = g1 ? -0.4238831152341712149578 : -0.2130139578384016019186;
                    const double p2d = g1 ? 0.2119415576170855242122 : 0.1065069789192007732037;
                    dfx = p1s * (fe - fw) + p1d * (fne - fnw) + p1d * (fse - fsw);
                    dfy = p1s * (fn - fs) + p1d * (fne - fse) + p1d * (fnw - fsw);
                    dfxx = p2c * fc + p2d1 * (fe + fw) + p2d2 * (fn + fs) + p2d * (fne + fnw + fsw + fse);
                    dfyy = p2c * fc + p2d2 * (fe + fw) + p2d1 * (fn + fs) + p2d * (fne + fnw + fsw + fse);
                    dfxy = 0.25 * (fne - fnw + fsw - fse);
                } else {
                    dfx = p2 * (fe - fw);
                    dfy = p2 * (fn - fs);
                    dfxx = fe - 2 * fc + fw;
                    dfyy = fn - 2 * fc + fs;
                    dfxy = 0.25 * (fne - fse - fnw + fsw);
                }
                fnew[IDX(y, x, q)] = fc - cxq * dfx - cyq * dfy + (cxxq * dfxx + cxyq * dfxy + cyyq * dfyy);
            }
        }
    }
}

/* stream_fdm_sofonea, src/fvm_bardow.F90:702-884: Lax-Wendroff along each
 * lattice direction, fu = f(x + c_q), fd = f(x - c_q). */
void oref_stream_fdm_sofonea(int nx, int ny, int ld, const double *fold, double *fnew, double dt)
{
    const double p2 = 0.5 / sqrt(2.0);
    /* :719 fnew(:,:,0) = fold(:,:,0) (all ld rows) */
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ld; y++) fnew[IDX(y, x, 0)] = fold[IDX(y, x, 0)];
    for (int q = 1; q <= 8; q++) {
        const int cxi = (int)CXD[q], cyi = (int)CYD[q];
#pragma omp parallel for schedule(static)
        for (int x1 = 1; x1 <= nx; x1++) {
            const int xp = xp1_of(x1, nx) - 1, xm = xm1_of(x1, nx) - 1, x = x1 - 1;
            for (int y1 = 1; y1 <= ny; y1++) {
                const int yp = xp1_of(y1, ny) - 1, ym = xm1_of(y1, ny) - 1, y = y1 - 1;
                const int xu = cxi > 0 ? xp : (cxi < 0 ? xm : x), xd = cxi > 0 ? xm : (cxi < 0 ? xp : x);
                const int yu = cyi > 0 ? yp : (cyi < 0 ? ym : y), yd = cyi > 0 ? ym : (cyi < 0 ? yp : y);
                const double fc = fold[IDX(y, x, q)], fu = fold[IDX(yu, xu, q)], fd = fold[IDX(yd, xd, q)];
                double du1, du2;
                if (q <= 4) {
                    du1 = 0.5 * (fu - fd);
                    du2 = fu - 2 * fc + fd;
                } else {
                    du1 = p2 * (fu - fd);
                    du2 = 0.5 * (fu - 2 * fc + fd);
                }
                fnew[IDX(y, x, q)] = fc + dt * (0.5 * dt * du2 - du1);
            }
        }
    }
}

/* perform_lbm_step with grid%streaming => stream_* (src/periodic_lbm.f90:15-29):
 * scheme 0 lbm_stream, 1 stream_fvm_bardow, 2/3/4 stream_fdm_bardow (central,
 * isotropic, least squares), 5 stream_fdm_sofonea. */
void oref_perform_step_scheme(int nx, int ny, int ld, double *f, int *iold, int *inew, int scheme, double dt,
                              int kind, double omega, double trt_magic, int nsteps)
{
    size_t lat = (size_t)ld * (size_t)nx * 9u;
    for (int s = 0; s < nsteps; s++) {
        double *fo = f + (size_t)(*iold - 1) * lat;
        double *fn = f + (size_t)(*inew - 1) * lat;
        switch (scheme) {
        case 1: oref_stream_fvm_bardow(nx, ny, ld, fo, fn, dt); break;
        case 2: case 3: case 4: oref_stream_fdm_bardow(nx, ny, ld, fo, fn, dt, scheme - 2); break;
        case 5: oref_stream_fdm_sofonea(nx, ny, ld, fo, fn, dt); break;
        case 6: case 7: oref_stream_fdm_bardow(nx, ny, ld, fo, fn, dt, scheme - 3); break;
        default: oref_lbm_stream(nx, ny, ld, fo, fn); break;
        }
        switch (kind) {
        case OREF_BGK: oref_collide_bgk(nx, ny, ld, fn, omega, 0); break;
        case OREF_TRT: oref_collide_trt(nx, ny, ld, fn, omega, oref_lambda_d(omega, trt_magic), 0); break;
        case OREF_RR: oref_collide_rr(nx, ny, ld, fn, omega); break;
        case OREF_BGKI: oref_collide_bgk_improved(nx, ny, fn, omega); break;
        default: break;
        }
        int t = *iold;
        *iold = *inew;
        *inew = t;
    }
}

/* ------------------------------------------------------------------------ */
/* src/benchmarks/taylor_green.f90:51-84 (t >= 0); arrays (ny,nx)            */
void oref_taylor_green_eval(int nx, int ny, double kx, double ky, double umax, double nu,
                            double t, double *p, double *ux, double *uy, int ref_loop)
{
    /* td from the constructor, src/benchmarks/taylor_green.f90:33 */
    double td = 1.0 / (nu * (kx * kx + ky * ky));
    int ylim = ref_loop ? nx : ny;
    for (int x1 = 1; x1 <= nx; x1++) {
        double xx = (double)(x1 - 1) + 0.5;
        for (int y1 = 1; y1 <= ylim; y1++) {
            double yy = (double)(y1 - 1) + 0.5;
            size_t o = (size_t)(y1 - 1) + (size_t)ny * (size_t)(x1 - 1);
            ux[o] = -umax * sqrt(ky / kx) * cos(kx * xx) * sin(ky * yy) * exp(-t / td);
            uy[o] = umax * sqrt(kx / ky) * sin(kx * xx) * cos(ky * yy) * exp(-t / td);
            p[o] = -0.25 * (umax * umax) * ((ky / kx) * cos(2.0 * kx * xx) + (kx / ky) * cos(2.0 * ky * yy)) *
                   exp(-2.0 * t / td);
        }
    }
}

/* src/benchmarks/shear_layer.f90:31-50; arrays (ny,nx) */
void oref_shear_layer_eval(int nx, int ny, double length, double u0, double k, double delta,
                           double rho0, double *rho, double *ux, double *uy)
{
    const double pi = 4.0 * atan(1.0);
    for (int x1 = 1; x1 <= nx; x1++) {
        double xd = ((double)(x1 - 1) + 0.5) / length;
        for (int y1 = 1; y1 <= ny; y1++) {
            double yd = ((double)(y1 - 1) + 0.5) / length;
            size_t o = (size_t)(y1 - 1) + (size_t)ny * (size_t)(x1 - 1);
            uy[o] = u0 * delta * sin(2.0 * pi * (xd + 0.25));
            if (yd <= 0.5) ux[o] = u0 * tanh(k * (yd - 0.25));
            else ux[o] = u0 * tanh(k * (0.75 - yd));
            rho[o] = rho0;
        }
    }
}

/* app/main_taylor_green.f90:195-202 */
double oref_tgv_l2_norm(int nx, int ny, const double *ux, const double *uy,
                        const double *uxa, const double *uya)
{
    double above = 0.0, below = 0.0;
    size_t n = (size_t)nx * (size_t)ny;
    for (size_t i = 0; i < n; i++) {
        double a = hypot(ux[i] - uxa[i], uy[i] - uya[i]);
        double b = hypot(uxa[i], uya[i]);
        above += a * a;
        below += b * b;
    }
    return sqrt(above) / sqrt(below);
}

double oref_kinetic_energy(int nx, int ny, const double *rho, const double *ux, const double *uy)
{
    double e = 0.0;
    for (int x = 0; x < nx; x++) {
        double col = 0.0;
        for (int y = 0; y < ny; y++) {
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            col += rho[o] * (ux[o] * ux[o] + uy[o] * uy[o]);
        }
        e += col;
    }
    return 0.5 * e;
}

/* ------------------------------------------------------------------------ */
/* Plugin semantics: sim/sim.F90                                             */
#define HIDX(i, j, q) ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (size_t)(q)))
static const double SW[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

/* sim/sim.F90:353-401 with ddf_shift = .true. */
static void sim_equilibrium(double rho, double ux, double uy, double feq[9])
{
    double uxx = ux * ux, uyy = uy * uy;
    double uxpy = ux + uy, uxmy = ux - uy;
    double indp = -1.5 * (uxx + uyy);
    feq[0] = W0 * rho * (indp);
    feq[1] = WS * rho * (indp + 3.0 * ux + 4.5 * uxx);
    feq[2] = WS * rho * (indp + 3.0 * uy + 4.5 * uyy);
    feq[3] = WS * rho * (indp - 3.0 * ux + 4.5 * uxx);
    feq[4] = WS * rho * (indp - 3.0 * uy + 4.5 * uyy);
    feq[5] = WD * rho * (indp + 3.0 * uxpy + 4.5 * uxpy * uxpy);
    feq[7] = WD * rho * (indp - 3.0 * uxpy + 4.5 * uxpy * uxpy);
    feq[6] = WD * rho * (indp - 3.0 * uxmy + 4.5 * uxmy * uxmy);
    feq[8] = WD * rho * (indp + 3.0 * uxmy + 4.5 * uxmy * uxmy);
    for (int q = 0; q < 9; q++) feq[q] = feq[q] + SW[q] * (rho - 1.0);
}

/* sim/sim.F90:181-199; p,u,v are (nx,ny) x fastest; f is (1-nh:nx+nh,1-nh:ny+nh,0:8) */
void oref_sim_eqinit_fields(int nx, int ny, int nhalo, double *f, const double *p,
                            const double *u, const double *v)
{
    size_t sx = (size_t)nx + 2u * (size_t)nhalo, sy = (size_t)ny + 2u * (size_t)nhalo;
    for (int j = 0; j < ny; j++) {
        for (int i = 0; i < nx; i++) {
            size_t o = (size_t)i + (size_t)nx * (size_t)j;
            double rho = 1.0 + p[o] / CSQR;
            double feq[9];
            sim_equilibrium(rho, u[o], v[o], feq);
            for (int q = 0; q < 9; q++)
                f[(size_t)(i + nhalo) + sx * ((size_t)(j + nhalo) + sy * (size_t)q)] = feq[q];
        }
    }
}

/* sim/sim.F90:148-179 */
void oref_sim_macros(int nx, int ny, int nhalo, const double *f, double *rho, double *u, double *v)
{
    size_t sx = (size_t)nx + 2u * (size_t)nhalo, sy = (size_t)ny + 2u * (size_t)nhalo;
    for (int j = 0; j < ny; j++) {
        for (int i = 0; i < nx; i++) {
            double fs[9];
            for (int q = 0; q < 9; q++) fs[q] = f[(size_t)(i + nhalo) + sx * ((size_t)(j + nhalo) + sy * (size_t)q)];
            size_t o = (size_t)i + (size_t)nx * (size_t)j;
            double r = (((fs[5] + fs[7]) + (fs[6] + fs[8])) + ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
            r = r + 1.0;
            rho[o] = r;
            u[o] = (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3])) / r;
            v[o] = (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4])) / r;
        }
    }
}

/* sim/sim.F90:404-505, push branch; halo lattices (0:nx+1,0:ny+1,0:8) */
void oref_sim_collide_stream_fused(int nx, int ny, const double *fsrc, double *fdst, double omega)
{
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; j++) {
        for (int i = 1; i <= nx; i++) {
            double fs[9], feq[9];
            for (int q = 0; q < 9; q++) fs[q] = fsrc[HIDX(i, j, q)];
            double rho = (((fs[5] + fs[7]) + (fs[6] + fs[8])) + ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
            rho = rho + 1.0;
            double ux = (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3])) / rho;
            double uy = (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4])) / rho;
            sim_equilibrium(rho, ux, uy, feq);
            fdst[HIDX(i, j, 0)] = omega * (feq[0] - fs[0]) + fs[0];
            fdst[HIDX(i + 1, j, 1)] = omega * (feq[1] - fs[1]) + fs[1];
            fdst[HIDX(i, j + 1, 2)] = omega * (feq[2] - fs[2]) + fs[2];
            fdst[HIDX(i - 1, j, 3)] = omega * (feq[3] - fs[3]) + fs[3];
            fdst[HIDX(i, j - 1, 4)] = omega * (feq[4] - fs[4]) + fs[4];
            fdst[HIDX(i + 1, j + 1, 5)] = omega * (feq[5] - fs[5]) + fs[5];
            fdst[HIDX(i - 1, j + 1, 6)] = omega * (feq[6] - fs[6]) + fs[6];
            fdst[HIDX(i - 1, j - 1, 7)] = omega * (feq[7] - fs[7]) + fs[7];
            fdst[HIDX(i + 1, j - 1, 8)] = omega * (feq[8] - fs[8]) + fs[8];
        }
    }
}

/* sim/sim.F90:568-624 (edges, then corners) */
void oref_sim_bc_push(int nx, int ny, double *f)
{
    for (int j = 1; j <= ny; j++) { /* EAST */
        f[HIDX(nx, j, 6)] = f[HIDX(0, j, 6)];
        f[HIDX(nx, j, 3)] = f[HIDX(0, j, 3)];
        f[HIDX(nx, j, 7)] = f[HIDX(0, j, 7)];
    }
    for (int j = 1; j <= ny; j++) { /* WEST */
        f[HIDX(1, j, 5)] = f[HIDX(nx + 1, j, 5)];
        f[HIDX(1, j, 1)] = f[HIDX(nx + 1, j, 1)];
        f[HIDX(1, j, 8)] = f[HIDX(nx + 1, j, 8)];
    }
    for (int i = 1; i <= nx; i++) { /* NORTH */
        f[HIDX(i, ny, 7)] = f[HIDX(i, 0, 7)];
        f[HIDX(i, ny, 4)] = f[HIDX(i, 0, 4)];
        f[HIDX(i, ny, 8)] = f[HIDX(i, 0, 8)];
    }
    for (int i = 1; i <= nx; i++) { /* SOUTH */
        f[HIDX(i, 1, 6)] = f[HIDX(i, ny + 1, 6)];
        f[HIDX(i, 1, 2)] = f[HIDX(i, ny + 1, 2)];
        f[HIDX(i, 1, 5)] = f[HIDX(i, ny + 1, 5)];
    }
    f[HIDX(nx, ny, 7)] = f[HIDX(0, 0, 7)];
    f[HIDX(nx, 1, 6)] = f[HIDX(0, ny + 1, 6)];
    f[HIDX(1, ny, 8)] = f[HIDX(nx + 1, 0, 8)];
    f[HIDX(1, 1, 5)] = f[HIDX(nx + 1, ny + 1, 5)];
}

/* sim/sim_slbm.F90:80-110 (gfortran branch: collide+push, bc, move_alloc swap).
 * On return f1 holds the current state, as after the reference's swap. */
void oref_sim_slbm_steps(int nx, int ny, double *f1, double *f2, double omega, int nsteps)
{
    size_t n = (size_t)(nx + 2) * (size_t)(ny + 2) * 9u;
    double *a = f1, *b = f2;
    for (int s = 0; s < nsteps; s++) {
        oref_sim_collide_stream_fused(nx, ny, a, b, omega);
        oref_sim_bc_push(nx, ny, b);
        double *t = a; a = b; b = t;
    }
    if (a != f1) {
        /* present the result in f1 and the previous state in f2, as move_alloc does */
        double *tmp = malloc(n * sizeof(double));
        memcpy(tmp, f1, n * sizeof(double));
        memcpy(f1, a, n * sizeof(double));
        memcpy(f2, tmp, n * sizeof(double));
        free(tmp);
    }
}

/* sim/sim_slbm.F90:198-205: norm2(u - ua) / norm2(ua) */
double oref_sim_norm(int nx, int ny, const double *u, const double *ua)
{
    double a = 0.0, b = 0.0;
    size_t n = (size_t)nx * (size_t)ny;
    for (size_t i = 0; i < n; i++) {
        double d = u[i] - ua[i];
        a += d * d;
        b += ua[i] * ua[i];
    }
    return sqrt(a) / sqrt(b);
}

/* ------------------------------------------------------------------------ */
/* Discrete adjoint of f_{n+1} = C(S(f_n)) (S = lbm_stream, C = collide_bgk),  */
/* f_0 = equilibrium(1, u0), u_T = j/rho of f_T.  New code, no reference      */
/* counterpart: the FP64 CPU check of the GPU adjoint.                        */
static const int CXA[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CYA[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const double WA[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

static void moments_u(const double g[9], double *rho, double *ux, double *uy)
{
    double r = 0.0, jx = 0.0, jy = 0.0;
    for (int q = 0; q < 9; q++) {
        r += g[q];
        jx += CXA[q] * g[q];
        jy += CYA[q] * g[q];
    }
    *rho = r;
    *ux = jx / r;
    *uy = jy / r;
}

static double *adj_states(int nx, int ny, const double *ux0, const double *uy0, double omega, int nsteps)
{
    int ld = oref_pad16(ny);
    size_t lat = (size_t)ld * (size_t)nx * 9u;
    double *F = calloc(lat * (size_t)(nsteps + 1), sizeof(double));
    double *one = malloc(sizeof(double) * (size_t)nx * (size_t)ny);
    for (size_t i = 0; i < (size_t)nx * (size_t)ny; i++) one[i] = 1.0;
    oref_set_pdf_to_equilibrium(nx, ny, ld, one, ux0, uy0, F);
    free(one);
    for (int n = 0; n < nsteps; n++) {
        oref_lbm_stream(nx, ny, ld, F + lat * (size_t)n, F + lat * (size_t)(n + 1));
        oref_collide_bgk(nx, ny, ld, F + lat * (size_t)(n + 1), omega, 0);
    }
    return F;
}

void oref_forward_bgk(int nx, int ny, const double *ux0, const double *uy0, double omega, int nsteps,
                      double *uxT, double *uyT)
{
    int ld = oref_pad16(ny);
    size_t lat = (size_t)ld * (size_t)nx * 9u;
    double *F = adj_states(nx, ny, ux0, uy0, omega, nsteps);
    const double *f = F + lat * (size_t)nsteps;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            double g[9], r;
            for (int q = 0; q < 9; q++) g[q] = f[IDX(y, x, q)];
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            moments_u(g, &r, &uxT[o], &uyT[o]);
        }
    free(F);
}

void oref_adjoint_bgk(int nx, int ny, const double *ux0, const double *uy0, double omega, int nsteps,
                      const double *gux, const double *guy, double *uxT, double *uyT,
                      double *grad_ux0, double *grad_uy0, double *grad_omega)
{
    int ld = oref_pad16(ny);
    size_t lat = (size_t)ld * (size_t)nx * 9u;
    double *F = adj_states(nx, ny, ux0, uy0, omega, nsteps);
    double *lam = calloc(lat, sizeof(double)), *nxt = calloc(lat, sizeof(double));
    /* lambda_T = dL/df_T = sum_a G_a (c_qa - u_a) / rho */
    const double *fT = F + lat * (size_t)nsteps;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            double g[9], r, u, v;
            for (int q = 0; q < 9; q++) g[q] = fT[IDX(y, x, q)];
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            moments_u(g, &r, &u, &v);
            uxT[o] = u;
            uyT[o] = v;
            for (int q = 0; q < 9; q++)
                lam[IDX(y, x, q)] = (gux[o] * (CXA[q] - u) + guy[o] * (CYA[q] - v)) / r;
        }
    double dom = 0.0;
    double *g = malloc(sizeof(double) * lat);
    for (int n = nsteps - 1; n >= 0; n--) {
        oref_lbm_stream(nx, ny, ld, F + lat * (size_t)n, g);
        memset(nxt, 0, sizeof(double) * lat);
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++) {
                double gg[9], feq[9], l[9], r, u, v;
                for (int q = 0; q < 9; q++) {
                    gg[q] = g[IDX(y, x, q)];
                    l[q] = lam[IDX(y, x, q)];
                }
                moments_u(gg, &r, &u, &v);
                oref_equilibrium(r, u, v, feq);
                double s0 = 0.0, A = 0.0, Bx = 0.0, By = 0.0, uu = u * u + v * v;
                for (int q = 0; q < 9; q++) {
                    dom += l[q] * (feq[q] - gg[q]);
                    double cu = CXA[q] * u + CYA[q] * v, wl = WA[q] * l[q];
                    s0 += wl;
                    A += wl * (1.0 - 4.5 * cu * cu + 1.5 * uu);
                    Bx += wl * (3.0 + 9.0 * cu) * CXA[q];
                    By += wl * (3.0 + 9.0 * cu) * CYA[q];
                }
                double ex = Bx - 3.0 * s0 * u, ey = By - 3.0 * s0 * v;
                for (int p = 0; p < 9; p++) {
                    double mu = (1.0 - omega) * l[p] + omega * (A + CXA[p] * ex + CYA[p] * ey);
                    int xs = (x - CXA[p] + nx) % nx, ys = (y - CYA[p] + ny) % ny; /* push along -c_p */
                    nxt[IDX(ys, xs, p)] = mu;
                }
            }
        double *t = lam; lam = nxt; nxt = t;
    }
    /* dL/du0 through f_0 = feq(1, u0) */
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            size_t o = (size_t)y + (size_t)ny * (size_t)x;
            double u = ux0[o], v = uy0[o], ax = 0.0, ay = 0.0;
            for (int q = 0; q < 9; q++) {
                double cu = CXA[q] * u + CYA[q] * v, wl = WA[q] * lam[IDX(y, x, q)];
                ax += wl * (3.0 * CXA[q] + 9.0 * cu * CXA[q] - 3.0 * u);
                ay += wl * (3.0 * CYA[q] + 9.0 * cu * CYA[q] - 3.0 * v);
            }
            grad_ux0[o] = ax;
            grad_uy0[o] = ay;
        }
    *grad_omega = dom;
    free(g); free(lam); free(nxt); free(F);
}
