/*
 * chem_oracle.c — CPU FP64 oracle of the REPROBUS chemistry step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (tests, smoke check,
 * CPU baseline of the benchmark). Never linked into the product library.
 *
 * PARITY UNPINNED: the reference has no tests or golden vectors and cannot be
 * compiled here (Fortran 77, no Fortran compiler in the image). This file
 * restates the reference routines statement by statement; every function
 * cites the lines of src/reprobus_l137_20230723.f ("F:") or src/jno.f90
 * ("JNO:") it follows.
 *
 * Fidelity rules kept throughout:
 *  - the reference is built with -r8: every REAL and every literal is FP64;
 *  - expressions keep the Fortran evaluation order (left to right within a
 *    precedence level), so that without FMA contraction (-ffp-contract=off)
 *    each operation rounds as the Fortran source says;
 *  - x**n with integer n is a product chain (x2=x*x, x3=x2*x, x4=x2*x2,
 *    x5=x3*x2, x6=x3*x3); x**r with real r is pow(x,r);
 *  - int()/aint() truncate toward zero;
 *  - max()/min() are fmax()/fmin() (NaN operands yield the other operand).
 * Deliberate deviation: hetero's K1S..K9S are zero-initialised (the reference
 * multiplies the uninitialised arrays by LNAT+LICE = 0, F:3397-3399,
 * F:3998-4026, which is NaN if the garbage is NaN).
 *
 * The work is done in blocks of nl longitudes of one latitude row; all loops
 * of chem3d are elementwise in (lon, level) except the vertical prefix sums of
 * total and jno, which run down whole columns, so blocking by longitude
 * reproduces the row computation exactly.
 */
#include "chem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/reprobus_chem.h"

#define NBCON 43
#define NCM 15
#define NPHOT 41
#define NZ 101
#define NSZA 27
#define NOZO 7

#define ORC_PI 3.141592653589793 /* 2.*asin(1.0), F:2750, F:5338 */

/* ---- global (Fortran-layout) array accessors, 0-based --------------------- */
#define G3(a, i, j, k) (a)[(size_t)(i) + (size_t)g->nlon * ((size_t)(j) + (size_t)g->nlat * (size_t)(k))]
#define G4(a, i, j, k, n) \
    (a)[(size_t)(i) + (size_t)g->nlon * ((size_t)(j) + (size_t)g->nlat * ((size_t)(k) + (size_t)g->niv * (size_t)(n)))]
#define GT(a, i, j, k, r) \
    (a)[(size_t)(i) + (size_t)g->nlon * ((size_t)(j) + (size_t)g->nlat * ((size_t)(k) + (size_t)g->niv * (size_t)(r)))]
/* arrays dimensioned (nlon,nlat,nivbas) */
#define GB(a, i, j, k) (a)[(size_t)(i) + (size_t)g->nlon * ((size_t)(j) + (size_t)g->nlat * (size_t)(k))]

/* rate-constant indices (order of F:930-1303) */
enum {
    K_a1, K_a1et, K_a2, K_a5, K_a6, K_a6b, K_a7, K_a17, K_a19, K_a26, K_a27, K_a30, K_a31, K_a36,
    K_b3, K_b4, K_b6, K_b7, K_b9, K_b12, K_b22, K_b23, K_b24, K_b27, K_b28, K_b32, K_b38, K_b39,
    K_c1a, K_c1b, K_c1c, K_c2, K_c3, K_c4, K_c5, K_c7, K_c8, K_c9, K_c10, K_c12, K_c14, K_c15,
    K_c17a, K_c17b, K_c18, K_c19,
    K_d2, K_d3, K_d4, K_d5, K_d6, K_d7, K_d8, K_d9, K_d10, K_d11, K_d31, K_d32, K_d33, K_d34,
    K_d35, K_d36, K_d37, K_d60, K_d61, K_d62, K_d90, K_d91, K_d92, K_d93, K_d94, K_d95, K_d96,
    K_d97,
    K_e2, K_e3, K_e4, K_e5a, K_e5b, K_e5c, K_e6, K_e7, K_e8, K_e9, K_e10, K_e11, K_e13, K_e15,
    K_e16, K_e50, K_e51, K_e52, K_e53, K_e54,
    K_hk1, K_hk2, K_hk3, K_hk4, K_hk5,
    K_COUNT
};

/* photolysis indices, F:754-794 (0-based) */
enum {
    J_o2, J_no2, J_o3_o1d, J_o3_o3p, J_no3_no, J_no3_no2, J_n2o5, J_hno3, J_hno4, J_h2o2,
    J_h2o, J_n2o, J_hocl, J_clono2_cl, J_clono2_clo, J_cl2o2, J_hcl, J_cl2, J_clno2, J_bro,
    J_brono2, J_hobr, J_oclo, J_brcl, J_ch3o2h, J_ch2o_hco, J_ch2o_co, J_cfc11, J_cfc12,
    J_cfc113, J_ccl4, J_ch3ccl3, J_ch3cl, J_hcfc22, J_ch3br, J_h1211, J_h1301, J_co2,
    J_ch2br2, J_hbr, J_no
};

/* ---- block workspace --------------------------------------------------------- */
typedef struct work {
    int nl, nb;          /* lons in block, chemistry levels */
    size_t n;            /* nl*nb */
    size_t nd;           /* n-sized double planes in base (4 int planes in ibase) */
    double* base;
    int* ibase;
    /* chem3d */
    double *t, *pm, *hnm, *n2, *o2, *co2, *h2, *ck0, *ck, *cc, *o3t, *sza, *tj, *het;
    double *parthno3, *parthno3sl, *parth2o, *parthcl, *parthbr, *vsed, *surf, *pr, *pe, *rk;
    double *rain_hno3, *rain_hno4, *rain_hcl, *rain_hbr, *rain_h2o2, *rain_ch2o, *rain_ch3o2h;
    double *day, *ch3o, *hco, *cc_prev, *ck_prev;
    /* analytic */
    double *parthno3l, *parthno3s, *dens, *ns, *pn0, *phcl0, *pw, *ms, *mn, *ws, *wn, *hhcl, *hhocl;
    double *hhobr, *hclono2, *hhbr, *tice, *aw, *wt, *mh2so4, *rmean, *aliq, *nnats, *nnatl, *anat;
    double *nice, *aice;
    int *lnat, *lice, *condliq;
    /* hetero */
    double *kl, *ks; /* 9 each */
    /* jno */
    double *colo2, *colno, *colo3, *pjno, *to3, *bd;
    /* phot */
    int *is;
} work;

static work* work_alloc(int nl, int nb) {
    work* w = (work*)calloc(1, sizeof(work));
    size_t n = (size_t)nl * nb;
    w->nl = nl;
    w->nb = nb;
    w->n = n;
    /* count of n-sized double arrays */
    size_t nd = 7 + NBCON + NBCON + NCM + 2 + NPHOT + 9 + 5 + 2 + NBCON + NBCON + K_COUNT + 7 + 3 + NCM +
                NBCON + 27 + 18 + 3 + 1 + 3 + 3;
    w->nd = nd;
    w->base = (double*)calloc(nd * n, sizeof(double));
    w->ibase = (int*)calloc(4 * n, sizeof(int));
    double* p = w->base;
#define TAKE(f, m) \
    do {           \
        w->f = p;  \
        p += (m) * n; \
    } while (0)
    TAKE(t, 1); TAKE(pm, 1); TAKE(hnm, 1); TAKE(n2, 1); TAKE(o2, 1); TAKE(co2, 1); TAKE(h2, 1);
    TAKE(ck0, NBCON); TAKE(ck, NBCON); TAKE(cc, NCM); TAKE(o3t, 1); TAKE(sza, 1); TAKE(tj, NPHOT);
    TAKE(het, 9); TAKE(parthno3, 1); TAKE(parthno3sl, 1); TAKE(parth2o, 1); TAKE(parthcl, 1);
    TAKE(parthbr, 1); TAKE(vsed, 1); TAKE(surf, 1); TAKE(pr, NBCON); TAKE(pe, NBCON); TAKE(rk, K_COUNT);
    TAKE(rain_hno3, 1); TAKE(rain_hno4, 1); TAKE(rain_hcl, 1); TAKE(rain_hbr, 1); TAKE(rain_h2o2, 1);
    TAKE(rain_ch2o, 1); TAKE(rain_ch3o2h, 1); TAKE(day, 1); TAKE(ch3o, 1); TAKE(hco, 1);
    TAKE(cc_prev, NCM); TAKE(ck_prev, NBCON);
    TAKE(parthno3l, 1); TAKE(parthno3s, 1); TAKE(dens, 1); TAKE(ns, 1); TAKE(pn0, 1); TAKE(phcl0, 1);
    TAKE(pw, 1); TAKE(ms, 1); TAKE(mn, 1); TAKE(ws, 1); TAKE(wn, 1); TAKE(hhcl, 1); TAKE(hhocl, 1);
    TAKE(hhobr, 1); TAKE(hclono2, 1); TAKE(hhbr, 1); TAKE(tice, 1); TAKE(aw, 1); TAKE(wt, 1);
    TAKE(mh2so4, 1); TAKE(rmean, 1); TAKE(aliq, 1); TAKE(nnats, 1); TAKE(nnatl, 1); TAKE(anat, 1);
    TAKE(nice, 1); TAKE(aice, 1);
    TAKE(kl, 9); TAKE(ks, 9);
    TAKE(colo2, 1); TAKE(colno, 1); TAKE(colo3, 1); TAKE(pjno, 1); TAKE(to3, 3); TAKE(bd, 3);
#undef TAKE
    w->lnat = w->ibase;
    w->lice = w->ibase + n;
    w->condliq = w->ibase + 2 * n;
    w->is = w->ibase + 3 * n;
    return w;
}

static void work_free(work* w) {
    if (!w) return;
    free(w->base);
    free(w->ibase);
    free(w);
}

/* A workspace of the m cells idx[0..m) of w: every per-cell plane is copied,
 * so a pass (which works cell by cell) gives on it what it gives on w. */
static work* work_subset(const work* w, const size_t* idx, size_t m) {
    work* s = work_alloc((int)m, 1);
    for (size_t p = 0; p < w->nd; p++)
        for (size_t j = 0; j < m; j++) s->base[p * m + j] = w->base[p * w->n + idx[j]];
    for (size_t p = 0; p < 4; p++)
        for (size_t j = 0; j < m; j++) s->ibase[p * m + j] = w->ibase[p * w->n + idx[j]];
    return s;
}

#define R(i, k) ((size_t)(i) + (size_t)nl * (size_t)(k))
#define S(arr, i, k, sp) (arr)[R(i, k) + w->n * (size_t)(sp)] /* species planes, 0-based sp */

/* ============================================================================
 * const, F:5927-5948
 * ========================================================================== */
void orc_const(double* troe) {
    troe[0] = 4.4e-32 * pow(300., 1.3);    /* a0hox  */
    troe[1] = 7.5e-11 * pow(300., -0.2);   /* a1hox  */
    troe[2] = 2.0e-30 * pow(300., 4.4);    /* a0nox1 */
    troe[3] = 1.4e-12 * pow(300., 0.7);    /* a1nox1 */
    troe[4] = 1.8e-30 * pow(300., 3.0);    /* a0nox2 */
    troe[5] = 2.8e-11 * pow(300., 0.0);    /* a1nox2 */
    troe[6] = 2.0e-31 * pow(300., 3.4);    /* a0nox3 */
    troe[7] = 2.9e-12 * pow(300., 1.1);    /* a1nox3 */
    troe[8] = 1.8e-31 * pow(300., 3.4);    /* a0clx1 */
    troe[9] = 1.5e-11 * pow(300., 1.9);    /* a1clx1 */
    troe[10] = 1.8e-31 * pow(300., 2.0);   /* a0clx2 */
    troe[11] = 1.0e-10 * pow(300., 1.0);   /* a1clx2 */
    troe[12] = 1.6e-32 * pow(300., 4.5);   /* a0clx3 */
    troe[13] = 3.0e-12 * pow(300., 2.0);   /* a1clx3 */
    troe[14] = 5.2e-31 * pow(300., 3.2);   /* a0brx  */
    troe[15] = 6.9e-12 * pow(300., 2.9);   /* a1brx  */
    troe[16] = 4.0e-31 * pow(300., 3.6);   /* a0c1   */
    troe[17] = 1.2e-12 * pow(300., -1.1);  /* a1c1   */
}

/* ============================================================================
 * total, F:5153-5186 — ozone column above each level (prefix sum from the top)
 * ========================================================================== */
static void orc_total(const orc_grid* g, const double* trajpre, int irapp, int ilat, int i0,
                      const double* hc, work* w) {
    const int nl = w->nl, nb = w->nb;
    const double zcmt = 2.120e20;
    for (int i = 0; i < nl; i++) w->o3t[R(i, 0)] = G4(hc, i0 + i, ilat, 0, 4) * w->hnm[R(i, 0)] * 6.8e5;
    for (int k = 1; k < nb; k++) {
        for (int i = 0; i < nl; i++) {
            double dp = (GT(trajpre, i0 + i, ilat, k, irapp) - GT(trajpre, i0 + i, ilat, k - 1, irapp)) * 100.;
            dp = fmax(dp, 0.);
            w->o3t[R(i, k)] =
                w->o3t[R(i, k - 1)] + zcmt * (G4(hc, i0 + i, ilat, k, 4) + G4(hc, i0 + i, ilat, k - 1, 4)) * .5 * dp;
        }
    }
}

/* ============================================================================
 * zenith, F:5308-5406
 * ========================================================================== */
static void orc_zenith(const orc_grid* g, const double* trajlon, const double* trajlat, int irapp, int ilat,
                       int i0, double day, work* w) {
    const int nl = w->nl, nb = w->nb;
    const double pi = ORC_PI;
    double ut = (day - trunc(day)) * 24.;
    double tz = 2. * pi * day / 365.;
    double sintz = sin(tz);
    double costz = cos(tz);
    double sin2tz = 2. * sintz * costz;
    double cos2tz = costz * costz - sintz * sintz;
    double sin3tz = sintz * cos2tz + costz * sin2tz;
    double cos3tz = costz * cos2tz - sintz * sin2tz;
    double rdecl = 0.006918 - 0.399912 * costz + 0.070257 * sintz - 0.006758 * cos2tz + 0.000907 * sin2tz -
                   0.002697 * cos3tz + 0.001480 * sin3tz;
    double eqr = 0.000075 + 0.001868 * costz - 0.032077 * sintz - 0.014615 * cos2tz - 0.040849 * sin2tz;
    double eqh = eqr * 24. / (2. * pi);
    for (int k = 0; k < nb; k++) {
        for (int i = 0; i < nl; i++) {
            double rlt = GT(trajlat, i0 + i, ilat, k, irapp) * pi / 180.;
            double lbut = 12. - eqh - GT(trajlon, i0 + i, ilat, k, irapp) * 24. / 360.;
            double lzut = 15. * (ut - lbut);
            double zpt = lzut * pi / 180.;
            double csz = sin(rlt) * sin(rdecl) + cos(rlt) * cos(rdecl) * cos(zpt);
            double zr = acos(csz);
            double s = zr * 180. / pi;
            w->sza[R(i, k)] = fmax(s, 0.);
        }
    }
}

/* ============================================================================
 * jno, JNO:1-249 — NO photolysis (Minschwaner & Siskind 1993)
 * ========================================================================== */
static const double JNO_SIGMA_O2[3][6] = {
    {1.12e-23, 2.45e-23, 7.19e-23, 3.04e-22, 1.75e-21, 1.11e-20},
    {1.35e-22, 2.99e-22, 7.33e-22, 3.07e-21, 1.69e-20, 1.66e-19},
    {2.97e-22, 5.83e-22, 2.05e-21, 8.19e-21, 4.80e-20, 2.66e-19}};
static const double JNO_SIGMA_NO_1[3][6] = {
    {0.00e+00, 1.32e-18, 6.35e-19, 7.09e-19, 2.18e-19, 4.67e-19},
    {0.00e+00, 0.00e+00, 3.05e-21, 5.76e-19, 2.29e-18, 2.21e-18},
    {1.80e-18, 1.50e-18, 5.01e-19, 7.20e-20, 6.72e-20, 1.49e-21}};
static const double JNO_SIGMA_NO_2[3][6] = {
    {0.00e+00, 4.41e-17, 4.45e-17, 4.50e-17, 2.94e-17, 4.35e-17},
    {0.00e+00, 0.00e+00, 3.20e-21, 5.71e-17, 9.09e-17, 6.00e-17},
    {1.40e-16, 1.52e-16, 7.00e-17, 2.83e-17, 2.73e-17, 6.57e-18}};
static const double JNO_W_NO_1[3][6] = {
    {0.00e+00, 5.12e-02, 1.36e-01, 1.65e-01, 1.41e-01, 4.50e-02},
    {0.00e+00, 0.00e+00, 1.93e-03, 9.73e-02, 9.75e-02, 3.48e-02},
    {4.50e-02, 1.80e-01, 2.25e-01, 2.25e-01, 1.80e-01, 4.50e-02}};
static const double JNO_W_NO_2[3][6] = {
    {0.00e+00, 5.68e-03, 1.52e-02, 1.83e-02, 1.57e-02, 5.00e-03},
    {0.00e+00, 0.00e+00, 2.14e-04, 1.08e-02, 1.08e-02, 3.86e-03},
    {5.00e-03, 2.00e-02, 2.50e-02, 2.50e-02, 2.00e-02, 5.00e-03}};
static const double JNO_DELTA_LAMBDA[3] = {2.3, 1.5, 1.5};
static const double JNO_I0[3] = {3.98e+11, 2.21e+11, 2.30e+11};
static const double JNO_SIGMA_O3[3] = {4.6e-19, 6.7e-19, 7.1e-19};

static void orc_jno(const double* cc_no, work* w, double* tjno) {
    const int nl = w->nl, nb = w->nb;
    const double factor = 3.141592 / 180.;
    const double zcmt = 287.0 / (1.38e-23 * 9.81);
    const double d = 1.65e+09, a = 5.1e+07, kq = 1.5e-09, r_o2 = 0.2095;
    const double* hnm = w->hnm;
    const double* o3t = w->o3t;
    const double* pm = w->pm;
    const double* sza = w->sza;
    for (int i = 0; i < nl; i++) {
        w->colo2[R(i, 0)] = 6.8e+05 * r_o2 * hnm[R(i, 0)];
        w->colno[R(i, 0)] = 6.8e+05 * cc_no[R(i, 0)];
        w->colo3[R(i, 0)] = o3t[R(i, 0)];
    }
    for (int k = 1; k < nb; k++) {
        for (int i = 0; i < nl; i++) {
            double dp = (pm[R(i, k)] - pm[R(i, k - 1)]) * 100.;
            dp = fmax(dp, 0.);
            w->colo2[R(i, k)] = w->colo2[R(i, k - 1)] + zcmt * (r_o2 + r_o2) * 0.5 * dp * 1.e-4;
            w->colno[R(i, k)] = w->colno[R(i, k - 1)] +
                                zcmt * (cc_no[R(i, k - 1)] / hnm[R(i, k - 1)] + cc_no[R(i, k)] / hnm[R(i, k)]) * 0.5 *
                                    dp * 1.e-4;
            w->colo3[R(i, k)] = o3t[R(i, k)];
        }
    }
    for (int k = 0; k < nb; k++) {
        for (int i = 0; i < nl; i++) {
            if (sza[R(i, 0)] <= 89.0) {
                double sec = 1. / cos(sza[R(i, 0)] * factor);
                w->colo2[R(i, k)] = w->colo2[R(i, k)] * sec;
                w->colno[R(i, k)] = w->colno[R(i, k)] * sec;
                w->colo3[R(i, k)] = w->colo3[R(i, k)] * sec;
                for (int b = 0; b < 3; b++)
                    w->to3[R(i, k) + w->n * b] = exp(-JNO_SIGMA_O3[b] * w->colo3[R(i, k)]);
                double n2 = hnm[R(i, k)] * 0.78;
                w->pjno[R(i, k)] = d / (a + d + kq * n2);
            }
        }
        for (int b = 0; b < 3; b++) {
            for (int i = 0; i < nl; i++) {
                if (sza[R(i, 0)] <= 89.0) {
                    double co2c = w->colo2[R(i, k)], cno = w->colno[R(i, k)];
                    double sum = 0.;
                    for (int s = 0; s < 6; s++) {
                        double term = exp(-JNO_SIGMA_O2[b][s] * co2c) *
                                      (JNO_W_NO_1[b][s] * JNO_SIGMA_NO_1[b][s] * exp(-JNO_SIGMA_NO_1[b][s] * cno) +
                                       JNO_W_NO_2[b][s] * JNO_SIGMA_NO_2[b][s] * exp(-JNO_SIGMA_NO_2[b][s] * cno));
                        sum = (s == 0) ? term : sum + term;
                    }
                    w->bd[R(i, k) + w->n * b] =
                        JNO_DELTA_LAMBDA[b] * JNO_I0[b] * w->to3[R(i, k) + w->n * b] * w->pjno[R(i, k)] * sum;
                    if (b == 2) {
                        tjno[R(i, k)] =
                            fmax(w->bd[R(i, k)] + w->bd[R(i, k) + w->n] + w->bd[R(i, k) + 2 * w->n], 1.e-30);
                    }
                }
            }
        }
    }
}

/* ============================================================================
 * phot, F:4996-5149 — trilinear interpolation of the J table
 * ========================================================================== */
static const double PHOT_DSZA[NSZA] = {0.,  5.,  10., 15., 20., 25., 30., 35., 40., 45., 50., 55., 60., 65.,
                                       70., 75., 80., 82., 84., 86., 88., 90., 91., 92., 93., 94., 95.};
static const double PHOT_XV3[NOZO] = {0.4, 0.6, 0.8, 1.0, 1.2, 1.4, 1.6};

#define AJL(nn, j, k, l) \
    g->ajl[(size_t)(nn) + (size_t)(NPHOT - 1) * ((size_t)(j) + (size_t)NZ * ((size_t)(k) + (size_t)NSZA * (size_t)(l)))]

static void orc_phot(const orc_grid* g, int ilat, int i0, const double* alt, work* w) {
    const int nl = w->nl, nb = w->nb;
    const double dz = 1.;
    double* tj = w->tj;
    for (size_t q = 0; q < (size_t)NPHOT * w->n; q++) tj[q] = 0.;
    for (int k = 0; k < nb; k++)
        for (int i = 0; i < nl; i++) w->is[R(i, k)] = NSZA - 1;
    for (int k = 0; k < nb; k++)
        for (int ii = 1; ii <= NSZA; ii++)
            for (int i = 0; i < nl; i++)
                if (PHOT_DSZA[ii - 1] >= w->sza[R(i, k)]) {
                    int c = ii - 1;
                    if (c < w->is[R(i, k)]) w->is[R(i, k)] = c;
                }
    const double stepo3 = (PHOT_XV3[NOZO - 1] - PHOT_XV3[0]) / (NOZO - 1);
    for (int k = nb - 1; k >= 0; k--) {
        for (int i = 0; i < nl; i++) {
            if (!(w->sza[R(i, k)] <= 95.)) continue;
            /* per-lon part of F:5078-5093 */
            double zin = G3(alt, i0 + i, ilat, k);
            zin = fmin(zin, 78.9);
            int iz = (int)(zin / dz) + 1;
            int ii = (int)zin;
            double v3std = g->o3up[ii] - (zin - (double)ii) * (g->o3up[ii] - g->o3up[ii + 1]);
            double v3rat = w->o3t[R(i, k)] / v3std;
            v3rat = fmax(v3rat, PHOT_XV3[0]);
            v3rat = fmin(v3rat, PHOT_XV3[NOZO - 1]);
            int iv = (int)trunc((v3rat - PHOT_XV3[0]) / stepo3) + 1;
            if (iv > NOZO - 1) iv = NOZO - 1;
            /* F:5096-5114 */
            int j = iz > 1 ? iz : 1;
            int kk = w->is[R(i, k)] > 1 ? w->is[R(i, k)] : 1;
            int l = iv > 1 ? iv : 1;
            double cizin = (zin - (double)(j - 1) * dz) / dz;
            double cisza = (w->sza[R(i, k)] - PHOT_DSZA[kk - 1]) / (PHOT_DSZA[kk] - PHOT_DSZA[kk - 1]);
            double cio3t = (v3rat - PHOT_XV3[l - 1]) / (PHOT_XV3[l] - PHOT_XV3[l - 1]);
            double w111 = (1. - cizin) * (1. - cisza) * (1. - cio3t);
            double w112 = (1. - cizin) * (1. - cisza) * cio3t;
            double w121 = (1. - cizin) * cisza * (1. - cio3t);
            double w122 = (1. - cizin) * cisza * cio3t;
            double w211 = cizin * (1. - cisza) * (1. - cio3t);
            double w212 = cizin * (1. - cisza) * cio3t;
            double w221 = cizin * cisza * (1. - cio3t);
            double w222 = cizin * cisza * cio3t;
            /* F:5117-5134 (1-based j,kk,l -> 0-based j-1, kk-1, l-1) */
            for (int nn = 0; nn < NPHOT - 1; nn++) {
                tj[R(i, k) + w->n * nn] =
                    w111 * AJL(nn, j - 1, kk - 1, l - 1) + w112 * AJL(nn, j - 1, kk - 1, l) +
                    w121 * AJL(nn, j - 1, kk, l - 1) + w122 * AJL(nn, j - 1, kk, l) +
                    w211 * AJL(nn, j, kk - 1, l - 1) + w212 * AJL(nn, j, kk - 1, l) +
                    w221 * AJL(nn, j, kk, l - 1) + w222 * AJL(nn, j, kk, l);
            }
        }
    }
    /* F:5146: J_NO from jno, with cc(:,:,8) = NO number density */
    orc_jno(w->cc + 7 * w->n, w, tj + (size_t)(NPHOT - 1) * w->n);
}

/* ============================================================================
 * density, F:4033-4073 — density of the ternary solution (g/cm3)
 * ========================================================================== */
static const double DENS_X[22] = {2.393284E-02, -4.359335E-05, 7.961181E-08, 0.0, -0.198716351, 1.39564574E-03,
                                  -2.020633E-06, 0.51684706, -3.0539E-03, 4.505475E-06, -0.30119511,
                                  1.840408E-03, -2.7221253742E-06, -0.11331674116, 8.47763E-04, -1.22336185E-06,
                                  0.3455282, -2.2111E-03, 3.503768245E-06, -0.2315332, 1.60074E-03,
                                  -2.5827835E-06};

static void orc_density(int nl, int kh, int kb, const double* ws, const double* wn, const double* temp,
                        double* dens) {
    const double* X = DENS_X - 1; /* 1-based */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            double T = temp[R(i, k)];
            double W = ws[R(i, k)] + wn[R(i, k)];
            double WH = 1.0 - W;
            double T2 = T * T, T3 = T2 * T;
            double V1 = X[1] + X[2] * T + X[3] * T2 + X[4] * T3;
            double VS = X[5] + X[6] * T + X[7] * T2 + (X[8] + X[9] * T + X[10] * T2) * W +
                        (X[11] + X[12] * T + X[13] * T2) * W * W;
            double VN = X[14] + X[15] * T + X[16] * T2 + (X[17] + X[18] * T + X[19] * T2) * W +
                        (X[20] + X[21] * T + X[22] * T2) * W * W;
            double VMCAL = WH / 18.0160 * V1 + VS * ws[R(i, k)] / 98.080 + VN * wn[R(i, k)] / 63.0160;
            dens[R(i, k)] = 1.0 / VMCAL * 0.001;
        }
    }
}

/* ============================================================================
 * hetero, F:3365-4029 — uptake coefficients -> second-order het rates
 * ========================================================================== */
static void orc_hetero(int nl, int kh, int kb, const double rice, const double rnats, const double rnatl,
                       work* w) {
    const double* temp = w->t;
    const double* ptot = w->pm;
    const double* hnm = w->hnm;
    double* K1L = w->kl + 0 * w->n; double* K2L = w->kl + 1 * w->n; double* K3L = w->kl + 2 * w->n;
    double* K4L = w->kl + 3 * w->n; double* K5L = w->kl + 4 * w->n; double* K6L = w->kl + 5 * w->n;
    double* K7L = w->kl + 6 * w->n; double* K8L = w->kl + 7 * w->n; double* K9L = w->kl + 8 * w->n;
    double* K1S = w->ks + 0 * w->n; double* K2S = w->ks + 1 * w->n; double* K3S = w->ks + 2 * w->n;
    double* K4S = w->ks + 3 * w->n; double* K5S = w->ks + 4 * w->n; double* K6S = w->ks + 5 * w->n;
    double* K7S = w->ks + 6 * w->n; double* K8S = w->ks + 7 * w->n; double* K9S = w->ks + 8 * w->n;
    /* deviation: zero-initialised (see header) */
    for (size_t q = 0; q < 9 * w->n; q++) w->ks[q] = 0.;

    /* ---- liquid aerosol, F:3436-3761 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            if (w->condliq[c] == 1) {
                double T = temp[c];
                double ZH2O = fmax(S(w->ck, i, k, 2), 1.E-08 * hnm[c]);
                double ZHCL = fmax(S(w->ck, i, k, 12), 1.E-13 * hnm[c]);
                double ZCLONO2 = fmax(S(w->ck, i, k, 13), 1.E-13 * hnm[c]);
                double ZHOCL = fmax(S(w->ck, i, k, 14), 1.E-13 * hnm[c]);
                double ZHOBR = fmax(S(w->ck, i, k, 25), 1.E-15 * hnm[c]);
                double ZHBR = fmax(S(w->ck, i, k, 18), 1.E-15 * hnm[c]);
                double phcl = (ZHCL / hnm[c]) * ptot[c] / 1013.;
                double pclono2 = (ZCLONO2 / hnm[c]) * ptot[c] / 1013.;
                double phocl = (ZHOCL / hnm[c]) * ptot[c] / 1013.;
                double phobr = (ZHOBR / hnm[c]) * ptot[c] / 1013.;
                double phbr = (ZHBR / hnm[c]) * ptot[c] / 1013.;
                (void)phocl;
                (void)phbr;
                double wt = w->wt[c];
                double wt2 = wt * wt, wt3 = wt2 * wt;
                double t0 = 144.11 + 0.166 * wt - 0.015 * wt2 + 2.18e-4 * wt3;
                double biga = 169.5 + 5.18 * wt - 0.0825 * wt2 + 3.27e-3 * wt3;
                double eta = biga * pow(T, -1.43) * exp(448. / (T - t0));
                double ah = exp(60.51 - 0.095 * wt + 0.0077 * wt2 - 1.61e-5 * wt3 - (1.76 + 2.52e-4 * wt2) * sqrt(T) +
                                (-805.89 + 253.05 * pow(wt, 0.076)) / sqrt(T));
                double dclono2 = 5.e-8 * T / eta;
                double cclono2 = 1474. * sqrt(T);
                double kh2o = 1.95e10 * exp(-2800. / T);
                double khh = 1.22e12 * exp(-6200. / T);
                double khydr = kh2o * w->aw[c] + khh * ah * w->aw[c];
                double gbh2o = 4 * w->hclono2[c] * 0.082 * T * sqrt(dclono2 * khydr) / cclono2;
                double mhcl = w->hhcl[c] * phcl;
                double khcl = 7.9e11 * ah * dclono2 * mhcl;
                double lclono2 = sqrt(dclono2 / (khydr + khcl));
                double fclono2 = 1. / tanh(w->rmean[c] / lclono2) - lclono2 / w->rmean[c];
                double grxn = fclono2 * gbh2o * sqrt(1. + khcl / khydr);
                double gbhcl = grxn * khcl / (khcl + khydr);
                double gs = 66.12 * w->hclono2[c] * mhcl * exp(-1374. / T);
                double fhcl = 1. / (1 + 0.612 * (gs + gbhcl) * pclono2 / phcl);
                double gps = fhcl * gs;
                double gbhclp = fhcl * gbhcl;
                double gb = gbhclp + grxn * khydr / (khcl + khydr);
                double gclono2 = 1. / (1. + 1. / (gps + gb));
                double gclono2hcl = gclono2 * (gps + gbhclp) / (gps + gb);
                double gclono2h2o = gclono2 - gclono2hcl;
                K1L[c] = 0.25 * gclono2h2o * cclono2 * w->aliq[c] / ZH2O;
                K2L[c] = 0.25 * gclono2hcl * cclono2 * w->aliq[c] / ZHCL;
                /* HOCl + HCl, F:3554-3578 */
                double chocl = 2009. * sqrt(T);
                double dhocl = 6.4e-8 * T / eta;
                double khoclhcl = 1.25e9 * ah * dhocl * mhcl;
                double lhocl = sqrt(dhocl / khoclhcl);
                double fhocl = 1. / tanh(w->rmean[c] / lhocl) - lhocl / w->rmean[c];
                grxn = 4. * w->hhocl[c] * 0.082 * T * sqrt(dhocl * khoclhcl) / chocl;
                double ghoclhcl = 1. / (1. + 1. / (fhocl * grxn * fhcl));
                K5L[c] = 0.25 * ghoclhcl * chocl * w->aliq[c] / ZHCL;
                /* HOBr + HCl, F:3590-3646 */
                double mhobr = w->hhobr[c] * phobr;
                double k2hobrhcl = exp(0.542 * wt - 6.44e3 / T + 10.3);
                double ratio = mhobr / mhcl;
                double rhobrhcl;
                if (ratio < 1.) {
                    double k1hobrhcl = k2hobrhcl * mhcl;
                    double dhobr = 6.2e-8 * T / eta;
                    double lhobr = sqrt(dhobr / k1hobrhcl);
                    double fhobr = 1. / tanh(w->rmean[c] / lhobr) - lhobr / w->rmean[c];
                    double chobr = 1477. * sqrt(T);
                    double ghobrhcl = 4. * w->hhobr[c] * 0.082 * T * sqrt(dhobr * k1hobrhcl) * fhobr / chobr;
                    rhobrhcl = 0.25 * ghobrhcl * chobr * w->aliq[c] / ZHCL;
                } else {
                    double k1hobrhcl = k2hobrhcl * mhobr;
                    double dhcl = 7.8e-8 * T / eta;
                    double lhcl = sqrt(dhcl / k1hobrhcl);
                    fhcl = 1. / tanh(w->rmean[c] / lhcl) - lhcl / w->rmean[c];
                    double chcl = 2408. * sqrt(T);
                    double ghobrhcl = 4. * w->hhcl[c] * 0.082 * T * sqrt(dhcl * k1hobrhcl) * fhcl / chcl;
                    rhobrhcl = 0.25 * ghobrhcl * chcl * w->aliq[c] / ZHOBR;
                }
                K7L[c] = rhobrhcl;
                K8L[c] = 0.;
                K9L[c] = 0.;
                /* N2O5 + H2O, F:3720-3724 */
                double GN2O5H2O = 0.1;
                double CBAR = 1400.1 * sqrt(T);
                K3L[c] = 0.25 * GN2O5H2O * CBAR * w->aliq[c] / ZH2O;
                K4L[c] = 0.;
                /* BrONO2 + H2O, F:3740-3746 */
                double gxrn = exp(29.24 - 0.396 * 100. * w->ws[c]) + 0.114;
                double gbrno3h2o = 1. / (1. / 0.805 + 1. / gxrn);
                CBAR = 1221.4 * sqrt(T);
                K6L[c] = 0.25 * gbrno3h2o * CBAR * w->aliq[c] / ZH2O;
            } else {
                K1L[c] = 0.; K2L[c] = 0.; K3L[c] = 0.; K4L[c] = 0.; K5L[c] = 0.;
                K6L[c] = 0.; K7L[c] = 0.; K8L[c] = 0.; K9L[c] = 0.;
            }
        }
    }
    /* ---- NAT, F:3763-3891 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            if (w->lnat[c] == 1) {
                double T = temp[c];
                double ZH2O = fmax(S(w->ck, i, k, 2), 1.E-08 * hnm[c]);
                double ZHCL = fmax(S(w->ck, i, k, 12), 1.E-13 * hnm[c]);
                const double GCLNO3HCLNAT = 0.2, GCLNO3H2ONAT = 0.004, GN2O5H2ONAT = 4.0E-4,
                             GN2O5HCLNAT = 3.0E-3, GHOCLHCLNAT = 0.1, GBRNO3H2ONAT = 0., GHOBRHCLNAT = 0.;
                const double P = ptot[c], NS = w->nnats[c], NL = w->nnatl[c];
#define NATR(G, M, Z)                                                                                 \
    ((G) * 4.56E4 * sqrt(T / (M)) * (rnats * rnats) * NS / (1.0 + 3.3E4 * (G) * rnats * P / T) / (Z) + \
     (G) * 4.56E4 * sqrt(T / (M)) * (rnatl * rnatl) * NL / (1.0 + 3.3E4 * (G) * rnatl * P / T) / (Z))
                K1S[c] = NATR(GCLNO3H2ONAT, 97.45, ZH2O);
                K2S[c] = NATR(GCLNO3HCLNAT, 97.45, ZHCL);
                K3S[c] = NATR(GN2O5H2ONAT, 108.0, ZH2O);
                K6S[c] = NATR(GBRNO3H2ONAT, 142.0, ZH2O);
                K4S[c] = NATR(GN2O5HCLNAT, 108.0, ZHCL);
                K5S[c] = NATR(GHOCLHCLNAT, 52.5, ZHCL);
                K7S[c] = NATR(GHOBRHCLNAT, 96.9, ZHCL);
#undef NATR
                K8S[c] = 0.;
                K9S[c] = 0.;
            }
        }
    }
    /* ---- ice, F:3893-3996 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            if (w->lice[c] == 1) {
                double T = temp[c];
                double ZH2O = fmax(S(w->ck, i, k, 2), 1.E-08 * hnm[c]);
                double ZHCL = fmax(S(w->ck, i, k, 12), 1.E-13 * hnm[c]);
                double ZHOBR = fmax(S(w->ck, i, k, 25), 1.E-13 * hnm[c]);
                const double GCLNO3HCLICE = 0.3, GCLNO3H2OICE = 0.3, GN2O5H2OICE = 0.02, GN2O5HCLICE = 0.03,
                             GHOCLHCLICE = 0.2, GBRNO3H2OICE = 0.3, GHOBRHCLICE = 0.3, GHOBRHBRICE = 0.1;
                const double P = ptot[c], NI = w->nice[c];
#define ICER(G, M, Z) ((G) * 4.56E4 * sqrt(T / (M)) * (rice * rice) * NI / (1.0 + 3.3E4 * (G) * rice * P / T) / (Z))
                K2S[c] = ICER(GCLNO3HCLICE, 97.45, ZHCL);
                K1S[c] = ICER(GCLNO3H2OICE, 97.45, ZH2O);
                K3S[c] = ICER(GN2O5H2OICE, 108.0, ZH2O);
                K4S[c] = ICER(GN2O5HCLICE, 108.0, ZHCL);
                K5S[c] = ICER(GHOCLHCLICE, 52.5, ZHCL);
                K6S[c] = ICER(GBRNO3H2OICE, 142.0, ZH2O);
                K7S[c] = ICER(GHOBRHCLICE, 96.9, ZHCL);
                K8S[c] = ICER(GHOBRHBRICE, 96.9, ZHOBR);
#undef ICER
            }
        }
    }
    /* ---- combine, F:3998-4026 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            double f = (double)(w->lnat[c] + w->lice[c]);
            for (int m = 0; m < 8; m++) w->het[c + w->n * m] = w->kl[c + w->n * m] + f * w->ks[c + w->n * m];
            w->het[c + w->n * 8] = 0.;
        }
    }
    (void)K9S;
}

/* ============================================================================
 * analytic, F:2620-3361 — PSC / liquid aerosol microphysics
 * ========================================================================== */
static const double AN_A1[3] = {12.37208932, 11.820654354, -180.06541028};
static const double AN_B1[3] = {-0.16125516114, -0.20786404244, -0.38601102592};
static const double AN_C1[3] = {-30.490657554, -4.807306373, -93.317846778};
static const double AN_D1[3] = {-2.1133114241, -5.1727540348, 273.88132245};
static const double AN_A2[3] = {13.455394705, 12.891938068, -176.95814097};
static const double AN_B2[3] = {-0.1921312255, -0.232338847708, -0.36257048154};
static const double AN_C2[3] = {-34.285174607, -6.4261237757, -90.469744201};
static const double AN_D2[3] = {-1.7620073078, -4.9005471319, 267.45509988};
static const double AN_BNRE[7] = {-3.18657, 0.992696, -0.153193e-2, -0.987059e-3, -0.578878e-3, 0.855176e-4,
                                  -0.327815e-5};
static const double AN_QN[10] = {14.5734, 0.0615994, -1.14895, 0.691693, -0.098863,
                                 0.0051579, 0.123472, -0.115574, 0.0110113, 0.0097914};
static const double AN_QS[10] = {14.4700, 0.0638795, -3.29597, 1.778224, -0.223244,
                                 0.0086486, 0.536695, -0.335164, 0.0265153, 0.0157550};
static const double AN_KN[7] = {-39.136, 6358.4, 83.29, -17650.0, 198.53, -11948, -28.469};
static const double AN_KS[7] = {-21.661, 2724.2, 51.81, -15732.0, 47.004, -6969.0, -4.6183};

static void orc_analytic(const orc_grid* g, int ilat, int i0, double* surfarea, work* w) {
    const int nl = w->nl, nb = w->nb;
    const int kh = g->nivhau - 1, kb = nb - 1; /* levels nivhau..nivbas */
    const double r = 8.205e-5, sigma = 1.8;
    const double* qn = AN_QN - 1;
    const double* qs = AN_QS - 1;
    const double* kn = AN_KN - 1;
    const double* ks = AN_KS - 1;
    const double* temp = w->t;
    const double* ptot = w->pm;
    const double* hnm = w->hnm;
    const double ndrop = 10.;
    const double nnat_small_max = 1.;
    const double rnats = 0.5e-4;
    const double rnatl = 6.5e-4;
    const double rice = 10.e-4;
    const double pi = ORC_PI;
    const double amu = 1.66e-24;
    double vnat = 0., vnatl = 0., vice = 0.;

    for (int k = 0; k < nb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            w->rmean[c] = 0.;
            w->aliq[c] = 0.;
            w->lnat[c] = 0;
            w->nnats[c] = 0.;
            w->nnatl[c] = 0.;
            w->anat[c] = 0.;
            w->lice[c] = 0;
            w->nice[c] = 0.;
            w->aice[c] = 0.;
            w->vsed[c] = 0.;
            w->condliq[c] = 0;
            w->parthno3[c] = 1.;
            w->parthno3l[c] = 1.;
            w->parthno3s[c] = 1.;
            w->parthno3sl[c] = 1.;
            w->parth2o[c] = 1.;
            w->parthcl[c] = 1.;
        }
    }
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            double qh2o = S(w->ck, i, k, 2) / hnm[c];
            w->pw[c] = qh2o * ptot[c] / 1013.0;
            w->pw[c] = fmin(w->pw[c], 2.e-3 / 1013.);
            double qhno3 = S(w->ck, i, k, 4) / hnm[c];
            w->pn0[c] = qhno3 * ptot[c] / 1013.0;
        }
    }
    /* ---- NAT, F:2795-2857 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            double t = fmin(temp[c], 273.);
            double pn0t = w->pn0[c] * 1013. * 0.75;
            double zmt = -2.7836 - 0.00088 * t;
            double zbt = 38.9855 - 11397.0 / t + 0.009179 * t;
            double zhno3eq = pow(10.0, zmt * log10(w->pw[c] * 1013. * 0.75) + zbt);
            if (pn0t / zhno3eq >= 1.) {
                w->lnat[c] = 1;
                double pn = zhno3eq / (0.75 * 1013.);
                double hno3s = (w->pn0[c] - pn) * 1013. * hnm[c] / ptot[c];
                hno3s = fmax(hno3s, 0.);
                vnat = hno3s * amu * 117. / 1.35;
                double vnat_small_max = nnat_small_max * (4. / 3. * pi * pow(rnats, 3.));
                if (vnat > vnat_small_max) {
                    w->nnats[c] = nnat_small_max;
                    w->nnatl[c] = (vnat - vnat_small_max) / (4. / 3. * pi * pow(rnatl, 3.));
                    vnatl = vnat - vnat_small_max;
                } else {
                    w->nnats[c] = vnat / (4. / 3. * pi * pow(rnats, 3.));
                    w->nnatl[c] = 0.;
                    vnatl = 0.;
                }
                w->anat[c] = w->nnats[c] * 4 * pi * (rnats * rnats) + w->nnatl[c] * 4 * pi * (rnatl * rnatl);
                w->parthno3s[c] = 1.0 - (w->pn0[c] - pn) / w->pn0[c];
                w->parthno3s[c] = fmax(w->parthno3s[c], 0.);
                w->parthno3s[c] = fmin(w->parthno3s[c], 1.);
                w->parthno3sl[c] = 1.0 - (w->pn0[c] - pn) * vnatl / vnat / w->pn0[c];
                w->parthno3sl[c] = fmax(w->parthno3sl[c], 0.);
                w->parthno3sl[c] = fmin(w->parthno3sl[c], 1.);
            }
        }
    }
    /* ---- ice, F:2861-2913 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            double t = fmin(temp[c], 273.);
            w->tice[c] = 2668.70 / (10.4310 - (log(w->pw[c]) + log(760.0)) / log(10.0));
            if (t <= w->tice[c]) {
                w->lice[c] = 1;
                w->lnat[c] = 0;
                w->anat[c] = 0.;
                double zh2oeq = pow(10.0, -2668.7 / t + 10.4310);
                double ph2o = zh2oeq / 760.0;
                double h2os = fmax(w->pw[c] - ph2o, 0.) * 1013. * hnm[c] / ptot[c];
                vice = h2os * amu * 18. / 0.928;
                w->nice[c] = vice / (4. / 3. * pi * pow(rice, 3.));
                w->aice[c] = w->nice[c] * 4 * pi * (rice * rice);
                w->parth2o[c] = 1.0 - fmax(w->pw[c] - ph2o, 0.) / w->pw[c];
                w->parth2o[c] = fmax(w->parth2o[c], 0.);
                w->parth2o[c] = fmin(w->parth2o[c], 1.);
                double zmt = -2.7836 - 0.00088 * t;
                double zbt = 38.9855 - 11397.0 / t + 0.009179 * t;
                double zhno3eq = pow(10.0, zmt * log10(w->pw[c] * w->parth2o[c] * 1013. * 0.75) + zbt);
                double pn = zhno3eq / (0.75 * 1013.);
                w->parthno3s[c] = 1.0 - (w->pn0[c] - pn) / w->pn0[c];
                w->parthno3s[c] = fmax(w->parthno3s[c], 0.);
                w->parthno3s[c] = fmin(w->parthno3s[c], 1.);
                w->parthno3sl[c] = w->parthno3s[c];
            }
        }
    }
    /* ---- liquid aerosols, F:2919-3056 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            w->condliq[c] = 1;
            double t = fmax(temp[c], fmax(w->tice[c] - 3.0, 185.));
            double qh2o = S(w->ck, i, k, 2) * w->parth2o[c] / hnm[c];
            w->pw[c] = qh2o * ptot[c] / 1013.0;
            w->pw[c] = fmin(w->pw[c], 2.e-3 / 1013.);
            w->pw[c] = fmax(w->pw[c], 2.e-5 / 1013.);
            double qh2so4 = fmax(S(w->ck, i, k, 11) / hnm[c], 1.e-18);
            w->ns[c] = ptot[c] * 100.0 * qh2so4 / 8.314 / t;
            double qhno3 = S(w->ck, i, k, 4) * w->parthno3s[c] / hnm[c];
            w->pn0[c] = ptot[c] / 1013.0 * qhno3;
            /* binary H2SO4/H2O */
            double a = ks[3] + ks[4] / t;
            double b = ks[1] + ks[2] / t;
            double cq = ks[5] + ks[6] / t + ks[7] * log(t) - log(w->pw[c]);
            double det = b * b - 4. * a * cq;
            double msb;
            if (det > 0.) {
                double xsb = (-b - sqrt(det)) / (2. * a);
                msb = 55.51 * xsb / (1.0 - xsb);
            } else {
                msb = 0.;
                w->condliq[c] = 0;
            }
            w->ms[c] = msb;
            w->ws[c] = msb * 0.098076 / (1.0 + msb * 0.098076);
            w->mn[c] = 0.0;
            w->wn[c] = 0.0;
            /* H2SO4 saturation pressure, F:2975-2988 */
            double wts = fmax(41., w->ws[c] * 100.);
            double wd = wts - 40.;
            double muh2so4 = 4.184 * (1.514e4 - 286. * wd + 1.08 * (wd * wd) - 3941. / pow(wd, 0.1));
            double ph2so4 = exp(-10156. / t + 16.2590 - muh2so4 / (8.314 * t));
            if (qh2so4 * ptot[c] / 1013. <= ph2so4) {
                w->ms[c] = 0.;
                w->ws[c] = 0.;
                w->condliq[c] = 0;
            }
            /* ternary HNO3/H2SO4/H2O, F:2994-3049 */
            if (w->condliq[c] == 1 && t < 215.) {
                double tf = t;
                double tt = r * tf * w->ns[c];
                double tr = 1.0e4 / tf - 43.4782608;
                double pr = log(w->pw[c]) + 18.4;
                double tr2 = tr * tr, tr3 = tr2 * tr, pr2 = pr * pr, pr3 = pr2 * pr;
                double hsb = qs[1] + qs[2] * tr2 + (qs[3] + qs[4] * tr + qs[5] * tr2 + qs[6] * tr3) * pr +
                             (qs[7] + qs[8] * tr + qs[9] * tr2) * pr2 + qs[10] * tr * pr3;
                hsb = exp(hsb);
                double kx = kn[1] + kn[2] / tf;
                double xnb = 1.0 / (2.0 * (kn[3] + kn[4] / tf)) *
                             (-kn[1] - kn[2] / tf -
                              pow(kx * kx - 4.0 * (kn[3] + kn[4] / tf) *
                                                (kn[5] + kn[6] / tf + kn[7] * log(tf) - log(w->pw[c])),
                                  0.5));
                double mnb = 55.51 * xnb / (1.0 - xnb);
                double hnb = qn[1] + qn[2] * tr2 + (qn[3] + qn[4] * tr + qn[5] * tr2 + qn[6] * tr3) * pr +
                             (qn[7] + qn[8] * tr + qn[9] * tr2) * pr2 + qn[10] * tr * pr3;
                hnb = exp(hnb);
                double mnb2 = mnb * mnb, msb2 = msb * msb;
                double pn0 = w->pn0[c];
                a = (tt * hnb * mnb2 - tt * hsb * mnb * msb - 2.0 * mnb2 * msb + mnb * msb2 + hnb * mnb * msb * pn0 -
                     hsb * msb2 * pn0) /
                    (mnb2 - mnb * msb);
                b = msb * (-(2.0 * tt * hnb * mnb) + tt * hsb * msb + mnb * msb - hnb * msb * pn0) / (mnb - msb);
                cq = (tt * hnb * mnb * msb2) / (mnb - msb);
                double a2 = a * a, a3 = a2 * a;
                double q = a2 - 3.0 * b;
                double q3 = q * q * q;
                double rr = -(2.0 * a3) + 9.0 * a * b - 27.0 * cq;
                double phi = atan(sqrt(fmax(4.0 * q3 - rr * rr, 0.)) / rr);
                if (phi < 0.) phi = phi + pi;
                double msf = -(1.0 / 3.0 * (a + 2.0 * sqrt(a2 - 3.0 * b) * cos((pi + phi) / 3.0)));
                msf = fmax(msf, 0.);
                double mnf = mnb * (1.0 - msf / msb);
                mnf = fmax(mnf, 0.);
                double pn = mnf / (hnb * mnf / (mnf + msf) + hsb * msf / (mnf + msf));
                double wsf = msf * 0.098076 / (1.0 + msf * 0.098076 + mnf * 0.063012);
                double wnf = mnf * 0.063012 / (1.0 + msf * 0.098076 + mnf * 0.063012);
                w->ms[c] = msf;
                w->mn[c] = mnf;
                w->ws[c] = wsf;
                w->wn[c] = wnf;
                w->parthno3l[c] = 1.0 - (w->pn0[c] - pn) / w->pn0[c];
                w->parthno3l[c] = fmin(w->parthno3l[c], 1.);
            }
            w->ws[c] = fmax(w->ws[c], 0.005);
        }
    }
    /* ---- density, F:3062 ---- */
    orc_density(nl, kh, kb, w->ws, w->wn, temp, w->dens);
    /* ---- volume, radius, area, solubilities, F:3068-3232 ---- */
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            if (w->condliq[c] == 1) {
                double vliq = w->ns[c] * 98.076e-6 / w->ws[c] / w->dens[c];
                double ls = log(sigma);
                double rmode = pow(3.0 * vliq / (4. * pi * ndrop) * exp(-9.0 / 2.0 * (ls * ls)), 1. / 3.);
                w->rmean[c] = rmode * exp(0.5 * (ls * ls));
                w->aliq[c] = 4.0 * pi * (rmode * rmode) * ndrop * exp(2.0 * (ls * ls));
                double t = fmax(temp[c], fmax(w->tice[c] - 3.0, 185.));
                double t2 = t * t, t3 = t2 * t;
                double ph2o0 = exp(18.452406985 - 3505.1578807 / t - 330918.55082 / t2 + 12725068.262 / t3);
                w->aw[c] = w->pw[c] * 1013. / ph2o0;
                w->aw[c] = fmin(w->aw[c], 1.);
                double y1, y2;
                double awc = w->aw[c];
                if (awc <= 0.05) {
                    y1 = AN_A1[0] * pow(awc, AN_B1[0]) + AN_C1[0] * awc + AN_D1[0];
                    y2 = AN_A2[0] * pow(awc, AN_B2[0]) + AN_C2[0] * awc + AN_D2[0];
                } else if (awc < 0.85) {
                    y1 = AN_A1[1] * pow(awc, AN_B1[1]) + AN_C1[1] * awc + AN_D1[1];
                    y2 = AN_A2[1] * pow(awc, AN_B2[1]) + AN_C2[1] * awc + AN_D2[1];
                } else {
                    y1 = AN_A1[2] * pow(awc, AN_B1[2]) + AN_C1[2] * awc + AN_D1[2];
                    y2 = AN_A2[2] * pow(awc, AN_B2[2]) + AN_C2[2] * awc + AN_D2[2];
                }
                double m = y1 + (t - 190.) * (y2 - y1) / 70.;
                w->wt[c] = 9800. * m / (98. * m + 1000.);
                w->wt[c] = fmax(w->wt[c], 0.5);
                w->mh2so4[c] = w->dens[c] * w->wt[c] / 9.8;
                double bigx = w->wt[c] / (w->wt[c] + (100. - w->wt[c]) * 98. / 18.);
                w->hhcl[c] = (0.094 - 0.61 * bigx + 1.2 * (bigx * bigx)) * exp(-8.68 + (8515. - 10718. * pow(bigx, 0.7)) / t);
                double qhcl = S(w->ck, i, k, 12) / hnm[c];
                w->phcl0[c] = qhcl * ptot[c] / 1013.0;
                double phcl1 = (w->phcl0[c] / (r * t)) / (1. / (r * t) + w->hhcl[c] * w->ns[c] / w->ms[c]);
                w->parthcl[c] = 1.0 - (w->phcl0[c] - phcl1) / w->phcl0[c];
                double sclono2 = 0.306 + 24. / t;
                w->hclono2[c] = 1.6e-6 * exp(4710. / t) * exp(-sclono2 * w->mh2so4[c]);
                double shocl = 0.0776 + 59.18 / t;
                w->hhocl[c] = 1.91e-6 * exp(5862.4 / t) * exp(-shocl * w->mh2so4[c]);
                w->hhobr[c] = 4.6e-4 * exp(4.5e3 / t);
                double wtc = w->wt[c];
                double mh2so4c = -1.977e-4 * (wtc * wtc) - 2.096e-2 * wtc + 4.445;
                double bh2so4 = -8.979e-5 * (wtc * wtc) + 2.141e-2 * wtc - 6.067;
                w->hhbr[c] = pow(10., mh2so4c * 1000. / t + bh2so4);
            }
        }
    }
    /* ---- total PSC area, F:3240-3246 ---- */
    for (int k = kh; k <= kb; k++)
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            w->surf[c] = w->aliq[c] + w->anat[c] * w->lnat[c] + w->aice[c] * w->lice[c];
            G3(surfarea, i0 + i, ilat, k) = w->surf[c];
        }
    /* ---- total HNO3 partition, F:3252-3258 ---- */
    for (int k = kh; k <= kb; k++)
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            w->parthno3[c] = w->parthno3l[c] * w->parthno3s[c];
            w->parthno3[c] = fmin(w->parthno3[c], 1.);
        }
    /* ---- settling velocity, F:3264-3348 ---- */
    const double rhoice = 0.928 * 1000.0;
    const double rhonat = 1.350 * 1000.0;
    for (int k = kh; k <= kb; k++) {
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            if (w->lice[c] == 1 || w->lnat[c] == 1) {
                double t = temp[c];
                double rpart = (w->lice[c] * rice + w->lnat[c] * rnatl) * 1.e-2;
                rpart = fmin(rpart, 535.e-6);
                if (rpart >= 0.5e-6) {
                    double rhopart = w->lice[c] * rhoice + w->lnat[c] * rhonat;
                    double rhoair = (hnm[c] * 28.97 / 6.022e23) * 1000.0;
                    double tcel = t - 273.15;
                    double netha = (1.718 + 0.0049 * tcel - 1.2e-5 * tcel * tcel) * 1.e-5;
                    double rp3 = rpart * rpart * rpart;
                    double cdnre2 = 32.0 * rp3 * (rhopart - rhoair) * rhoair * 9.80665 / (3.0 * (netha * netha));
                    double L = log(cdnre2);
                    double L2 = L * L, L3 = L2 * L, L4 = L2 * L2, L5 = L3 * L2, L6 = L3 * L3;
                    double ynre = AN_BNRE[0] + AN_BNRE[1] * L + AN_BNRE[2] * L2 + AN_BNRE[3] * L3 + AN_BNRE[4] * L4 +
                                  AN_BNRE[5] * L5 + AN_BNRE[6] * L6;
                    double nre = exp(ynre);
                    if (nre >= 1.e-2) {
                        w->vsed[c] = netha * nre / (2 * rhoair * rpart);
                    } else {
                        double lambda0 = 6.6e-8;
                        double lambda = lambda0 * (1013.25 / ptot[c]) * (t / 293.15);
                        double us = 2.0 * (rpart * rpart) * 9.80665 * (rhopart - rhoair) / (9.0 * netha);
                        double shapek = 1.2;
                        double vsedsol = us / shapek *
                                         (1.0 + 1.246 * lambda / rpart + 0.42 * lambda / rpart * exp(-(0.87 * rpart / lambda)));
                        w->vsed[c] = vsedsol;
                    }
                }
            }
        }
    }
    /* ---- hetero, F:3354 ---- */
    orc_hetero(nl, kh, kb, rice, rnats, rnatl, w);
    (void)vnat;
    (void)vice;
}

/* ============================================================================
 * chem3d rate constants, F:920-1306
 * ========================================================================== */
static void orc_rates(const orc_grid* g, work* w) {
    const size_t n = w->n;
    const double xln6 = log(0.6);
    const double* tr = g->troe;
    const double a0hox = tr[0], a1hox = tr[1], a0nox1 = tr[2], a1nox1 = tr[3], a0nox2 = tr[4], a1nox2 = tr[5],
                 a0nox3 = tr[6], a1nox3 = tr[7], a0clx1 = tr[8], a1clx1 = tr[9], a0clx2 = tr[10], a1clx2 = tr[11],
                 a0clx3 = tr[12], a1clx3 = tr[13], a0brx = tr[14], a1brx = tr[15], a0c1 = tr[16], a1c1 = tr[17];
    for (size_t c = 0; c < n; c++) {
        double* K = w->rk;
#define RK(name) K[(size_t)K_##name * n + c]
        const double t = w->t[c];
        const double hnm = w->hnm[c];
        const double pm = w->pm[c];
        double lntemp = log(t);
        double ak0, ak1, rate, xpo, deq, l10;
#define TROE(A0, E0, A1, E1, OUT)                    \
    ak0 = (A0) * exp(lntemp * (E0));                 \
    ak1 = (A1) * exp(lntemp * (E1));                 \
    rate = (ak0 * hnm) / (1. + ak0 * hnm / ak1);     \
    l10 = log10((ak0 * hnm) / ak1);                  \
    xpo = 1. / (1. + l10 * l10);                     \
    OUT = rate * exp(xln6 * xpo)
        TROE(a0hox, -1.3, a1hox, 0.2, RK(a1));
        RK(a1et) = 1.63e-10 * exp(60. / t);
        RK(a2) = 1.4e-10 * exp(-470. / t);
        RK(a5) = 1.8e-11 * exp(180. / t);
        RK(a6) = 1.7e-12 * exp(-940. / t);
        RK(a6b) = 1.0e-14 * exp(-490. / t);
        RK(a7) = 3.0e-11 * exp(200. / t);
        RK(a17) = 4.8e-11 * exp(250. / t);
        RK(a19) = 2.8e-12 * exp(-1800. / t);
        RK(a26) = 3.3e-12 * exp(270. / t);
        RK(a27) = 1.5e-12 * exp(19. / t) + 2.1e-33 * exp(920. / t) * hnm;
        RK(a30) = 1.8e-12;
        RK(a31) = 1.8e-12;
        RK(a36) = 1.5e-13 * (1. + .6 * pm / 1013.);
        RK(b3) = 5.1e-12 * exp(210. / t);
        RK(b4) = 3.0e-12 * exp((-1500. / t));
        RK(b6) = 2.1e-11 * exp((100. / t));
        RK(b7) = 1.5e-11 * exp((-3600. / t));
        RK(b9) = 1.2e-13 * exp((-2450. / t));
        TROE(a0nox1, -4.4, a1nox1, -0.7, RK(b12));
        TROE(a0nox2, -3.0, a1nox2, 0.0, RK(b22));
        TROE(a0nox3, -3.4, a1nox3, -1.1, RK(b23));
        deq = 2.1e-27 * exp(10900. / t);
        RK(b24) = RK(b23) / (deq * hnm);
        {
            double aux1 = 2.7e-17 * exp(2199. / t);
            double aux2 = 1. + aux1 / (6.5e-34 * exp(1335. / t) * hnm);
            RK(b27) = 2.4e-14 * exp(460. / t) + aux1 / aux2;
        }
        RK(b28) = 1.3e-12 * exp(380. / t);
        deq = 2.7e-27 * exp(11000. / t);
        RK(b32) = RK(b12) / (deq * hnm);
        RK(b38) = 4.63e-11 * exp(20. / t);
        RK(b39) = 7.25e-11 * exp(20. / t);
        RK(c1a) = 1.31e-10;
        RK(c1b) = 0.35e-10;
        RK(c1c) = 0.09e-10;
        RK(c2) = 2.45e-12 * exp((-1775. / t));
        RK(c3) = 1.1e-10;
        TROE(a0c1, -3.6, a1c1, 1.1, RK(c4));
        RK(c5) = 2.8e-12 * exp((300. / t));
        RK(c7) = 3.8e-13 * exp((800. / t));
        RK(c8) = 5.5e-12 * exp(125. / t);
        RK(c9) = 3.4e-11 * exp((-1600. / t));
        RK(c10) = 8.1e-11 * exp((-30. / t));
        RK(c12) = 5.2e-12;
        RK(c14) = 9.5e-14 * exp((390. / t));
        RK(c15) = 3.9e-14 * exp((-900. / t));
        RK(c17a) = 3.8e-12 * exp((200. / t)) * 0.7;
        RK(c17b) = 3.8e-12 * exp((200. / t)) * 0.3;
        RK(c18) = 3.3e-12 * exp((-115. / t));
        RK(c19) = 1.7e-11 * exp((-800. / t));
        RK(d2) = 2.3e-11 * exp((-200. / t));
        RK(d3) = 2.8e-11 * exp(85. / t);
        RK(d4) = 6.4e-12 * exp(290. / t);
        RK(d5) = 7.3e-12 * exp((-1280. / t));
        RK(d6) = 3.05e-11 * exp((-2270. / t));
        RK(d7) = 1.4e-11 * exp(269. / t);
        RK(d8) = 7.4e-12 * exp(270. / t);
        RK(d9) = 6.0e-13 * exp(230. / t);
        RK(d10) = 3.6e-11 * exp(-375. / t);
        RK(d11) = 1.8e-12 * exp((-250. / t));
        TROE(a0clx1, -3.4, a1clx1, -1.9, RK(d31));
        RK(d32) = 3.6e-12 * exp((-840. / t));
        RK(d33) = 2.6e-12 * exp(290. / t);
        RK(d34) = 3.0e-12 * exp((-500. / t));
        RK(d35) = 1.7e-13;
        TROE(a0clx2, -2., a1clx2, -1., RK(d36));
        RK(d37) = 3.4e-12 * exp((-130. / t));
        TROE(a0clx3, -4.5, a1clx3, -2.0, RK(d60));
        deq = 1.72e-27 * exp(8649. / t);
        RK(d61) = RK(d60) / (deq * hnm);
        RK(d62) = 1.0e-12 * exp(-1590. / t) + 3.0e-11 * exp(-2450. / t);
        RK(d90) = 2.3e-10;
        RK(d91) = 1.4e-10;
        RK(d92) = 2.0e-10;
        RK(d93) = 3.3e-10;
        RK(d94) = 1.64e-12 * exp((-1520. / t));
        RK(d95) = 2.4e-12 * exp((-1250. / t));
        RK(d96) = 1.0e-10;
        RK(d97) = 1.05e-12 * exp((-1600. / t));
        RK(e2) = 1.6e-11 * exp((-780. / t));
        RK(e3) = 1.9e-11 * exp(230. / t);
        RK(e4) = 8.8e-12 * exp(260. / t);
        RK(e5a) = 9.5e-13 * exp(550. / t);
        RK(e5b) = 2.3e-12 * exp(260. / t);
        RK(e5c) = 4.1e-13 * exp(290. / t);
        RK(e6) = 1.5e-12 * exp(230. / t);
        RK(e7) = 4.8e-12 * exp(-310. / t);
        RK(e8) = 1.9e-11 * exp(215. / t);
        RK(e9) = 1.5e-10;
        RK(e10) = 1.7e-11 * exp(250. / t);
        RK(e11) = 5.5e-12 * exp(200. / t);
        TROE(a0brx, -3.2, a1brx, -2.9, RK(e13));
        RK(e15) = 4.5e-12 * exp(460. / t);
        RK(e16) = 1.2e-10 * exp((-430. / t));
        RK(e50) = 1.8e-10;
        RK(e51) = 2.35e-12 * exp((-1300. / t));
        RK(e52) = 1.5e-10;
        RK(e53) = 1.0e-10;
        RK(e54) = 2.0e-12 * exp(-840. / t);
        RK(hk1) = 4.23e-28 * hnm / (t * t);
        RK(hk2) = 6.0e-34 * pow(300. / t, 2.4) * hnm;
        RK(hk3) = 8.e-12 * exp((-2060. / t));
        RK(hk4) = 2.15e-11 * exp(110. / t);
        RK(hk5) = 3.3e-11 * exp(55. / t);
#undef TROE
#undef RK
    }
}

/* ============================================================================
 * chem3d iteration body (one pass), F:1350-2372
 * ========================================================================== */
static void orc_pass(const orc_grid* g, double dt, work* w) {
    const size_t n = w->n;
    const double a3et = 1.2e-10, a23a = 7.2e-11, a23b = 6.9e-12, a23c = 1.6e-12;
    for (size_t c = 0; c < n; c++) {
#define K(name) w->rk[(size_t)K_##name * n + c]
#define CK(m) w->ck[(size_t)((m)-1) * n + c]
#define CC(m) w->cc[(size_t)((m)-1) * n + c]
#define TJ(name) w->tj[(size_t)(J_##name) * n + c]
#define HET(m) w->het[(size_t)((m)-1) * n + c]
        const double o2 = w->o2[c], n2 = w->n2[c], h2 = w->h2[c], hnm = w->hnm[c];
        const double parthno3 = w->parthno3[c], parth2o = w->parth2o[c], parthcl = w->parthcl[c],
                     parthbr = w->parthbr[c];
        double a, b;
        if (w->sza[c] <= 95.) {
            /* ---- day, F:1357-1665 ---- */
            w->day[c] = 1.;
            CC(15) = ((K(c2) * CC(2) + K(c1a) * CC(1) + K(d5) * CC(3)) * CK(2)) / (K(c4) * o2 + K(c3) * CC(4));
            w->ch3o[c] = (K(c1b) * CC(1) * CK(2) + (K(c5) * CC(8) + 2. * K(c14) * CK(29) + K(c18) * CC(11)) * CK(29) +
                          TJ(ch3o2h) * CK(30)) /
                         (K(c15) * o2);
            w->hco[c] = (K(c8) * CC(2) + K(c9) * CC(4) + K(c10) * CC(3) + K(c19) * CC(9) + TJ(ch2o_hco)) * CK(28) /
                        (K(c12) * o2);
            double r1 = (TJ(o3_o1d) + TJ(o3_o3p) + K(a2) * CC(14) + K(a6) * CC(2) + K(a6b) * CC(6) + K(b4) * CC(8) +
                         K(d2) * CC(3)) /
                        (K(hk2) * o2);
            double r2 = 1. / (1. + r1);
            CC(5) = r2 * CK(8);
            CC(4) = r1 * CC(5);
            double r3 = TJ(o3_o1d) / (K(hk4) * n2 + K(hk5) * o2);
            CC(1) = r3 * CC(5);
            double r4 = (K(a5) * CC(4) + K(a36) * CK(9) + K(a19) * h2) /
                        (K(a1) * o2 + K(a2) * CC(5) + (a23a + a23b + a23c) * CC(6));
            CC(14) = r4 * CC(2);
            double r7 = TJ(no) / (K(b7) * o2 + K(b6) * CC(8));
            double r8 = (K(b9) * CC(5)) / (TJ(no3_no) + TJ(no3_no2) + K(b12) * CC(7));
            double r5 = (TJ(no2) + K(b3) * CC(4) + TJ(no3_no) * r8) /
                        (K(b4) * CC(5) + K(a26) * CC(6) + K(d4) * CC(11) + K(e4) * CC(12) + K(c5) * CK(29));
            CC(7) = CK(21) / (1. + r5 + r7 * r5 + r8);
            CC(8) = r5 * CC(7);
            CC(10) = r7 * CC(8);
            CC(13) = r8 * CC(7);
            double r6 = (K(a6) * CC(5) + K(a30) * CK(17) + K(c8) * CK(28) + K(d8) * CC(11) + K(e10) * CC(12) +
                         K(a1) * o2 * r4) /
                        ((a23a + a23b + a23c) * CC(14) + K(a6b) * CC(5) + K(a7) * CC(4) + K(a26) * CC(8) +
                         2. * K(a27) * CC(6) + K(a17) * CC(2) + K(d7) * CC(3) + K(d10) * CC(3) + K(d33) * CC(11) +
                         K(e7) * CC(9) + K(e15) * CC(12));
            a = .5;
            b = 1. - a;
            CC(6) = a * CC(6) + b * CC(2) * r6;
            double r13 = K(d31) * CC(7) /
                         (TJ(clono2_cl) + TJ(clono2_clo) + K(d32) * CC(4) + HET(1) * CK(3) + HET(2) * CK(13));
            double r9 = (K(d33) * CC(6) + HET(1) * CK(3) * r13) / (HET(5) * CK(13) + K(d35) * CC(4) + TJ(hocl));
            double r10 = (K(d60) * CC(11)) / (K(d61) * hnm + TJ(cl2o2));
            double r12 = K(e5c) * CC(12) / TJ(brcl);
            double r11 = (K(d3) * CC(4) + K(d4) * CC(8) + K(d8) * CC(2) + K(c18) * CK(29) + K(e5b) * CC(12) +
                          TJ(clono2_cl) * r13 + TJ(hocl) * r9 + 2. * TJ(cl2o2) * r10 + TJ(brcl) * r12) /
                         (K(d2) * CC(5) + K(d5) * CK(2) + K(d7) * CC(6) + K(d10) * CC(6) + K(d37) * CK(15));
            a = .5;
            b = 1. - a;
            CC(11) = a * CC(11) + b * CK(23) / (1. + r11);
            CC(3) = r11 * CC(11);
            double r27 = K(e13) * CC(7) / (TJ(brono2) + K(e8) * CC(4));
            double r28 = K(e15) * CC(6) / (TJ(hobr) + K(e16) * CC(4));
            double r29 = K(e5c) * CC(11) / TJ(brcl);
            double r30 = (K(e3) * CC(4) + K(e4) * CC(8) + K(e5a) * CC(11) + K(e5b) * CC(11) + 2. * K(e6) * CC(12) +
                          K(e10) * CC(2) + TJ(bro) + TJ(brono2) * 0.85 * r27 + TJ(hobr) * r28 + TJ(brcl) * r29) /
                         (K(e2) * CC(5) + K(e7) * CC(6) + K(c19) * CK(28));
            a = .5;
            b = 1. - a;
            CC(12) = a * CC(12) + b * CK(24) / (1. + r30);
            CC(9) = r30 * CC(12);
            double coea = 2. * K(a31) + 2. * (K(a17) + K(a27) * r6 + (a23b + a23c) * r4) * r6;
            double coeb = K(b27) * CK(5) * parthno3 + K(b22) * CC(7) + K(b28) * CK(22) + K(b23) * CC(7) * r6 +
                          K(c2) * CK(2) + K(c7) * CK(29) * r6 + K(c8) * CK(28) + K(c17a) * CK(30) +
                          K(d7) * CC(3) * r6 + K(d9) * CC(11) + K(d11) * CK(13) * parthcl + K(d33) * CC(11) * r6 +
                          K(d34) * CK(15) + K(e11) * CK(19) * parthbr + K(e7) * CC(9) * r6 + K(e15) * CC(12) * r6;
            double t01 = 2. * (K(a1et) * CC(1) + TJ(h2o)) * CK(3) * parth2o;
            double t02 = ((K(c1a) + K(c1b)) * CK(2) + 2. * a3et * h2) * CC(1);
            double t03 = K(c3) * CC(15) * CC(4);
            double t04 = TJ(ch3o2h) * CK(30);
            double t05 = K(c15) * w->ch3o[c] * o2;
            double t06 = (TJ(ch2o_hco) + K(c9) * CC(4)) * CK(28);
            double t07 = K(c12) * w->hco[c] * o2;
            double t08 = TJ(hno3) * CK(5) * parthno3;
            double t09 = (K(b24) * hnm + TJ(hno4)) * CK(22);
            double t10 = (K(d35) * CC(4) + K(d37) * CC(3) + TJ(hocl)) * CK(15);
            double t11 = 2. * TJ(h2o2) * CK(17);
            double t12 = K(d6) * h2 * CC(3);
            double t13 = TJ(hobr) * CK(26);
            double t14 = K(e16) * CC(4) * CK(26);
            double t15 = TJ(hbr) * CK(19);
            double coec = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13 + t14 + t15;
            double argum = coeb * coeb + 4. * coea * coec;
            argum = fmax(argum, 0.);
            a = .5;
            b = 1. - a;
            CC(2) = a * CC(2) + b * (sqrt(argum) - coeb) / (2. * coea);
        } else {
            /* ---- night, F:1673-1746 ---- */
            w->day[c] = 0.;
            CC(14) = 0.;
            CC(15) = 0.;
            w->ch3o[c] = 0.;
            w->hco[c] = 0.;
            CC(1) = 0.;
            CC(4) = 0.;
            CC(5) = CK(8);
            CC(2) = 0.;
            CC(3) = 0.;
            CC(6) = 0.;
            CC(8) = 0.;
            double r8 = K(b9) * CC(5) / (K(b12) * fmax(CC(7), 1.e-30));
            CC(7) = CK(21) / (1. + r8);
            CC(13) = r8 * CC(7);
            CC(10) = 0.;
            CC(11) = fmax(CK(23), 0.);
            CC(9) = 0.;
            CC(12) = fmax(CK(24), 0.);
        }
    }
    /* ---- production / loss, F:1758-2358 ---- */
    for (size_t c = 0; c < n; c++) {
        const double o2 = w->o2[c], h2 = w->h2[c], hnm = w->hnm[c], co2 = w->co2[c];
        const double parthno3 = w->parthno3[c], parth2o = w->parth2o[c], parthcl = w->parthcl[c],
                     parthbr = w->parthbr[c];
        const double day = w->day[c], ch3o = w->ch3o[c], hco = w->hco[c];
        const double rain_hno3 = w->rain_hno3[c], rain_hno4 = w->rain_hno4[c], rain_hcl = w->rain_hcl[c],
                     rain_hbr = w->rain_hbr[c], rain_h2o2 = w->rain_h2o2[c], rain_ch2o = w->rain_ch2o[c],
                     rain_ch3o2h = w->rain_ch3o2h[c];
#define PR(m) w->pr[(size_t)((m)-1) * n + c]
#define PE(m) w->pe[(size_t)((m)-1) * n + c]
        double t01, t02, t03, t04, t05, t06, t07, t08, t09, t10, t11, t12, t13, t14;
        /* n2o */
        PR(1) = 0.e0;
        PE(1) = TJ(n2o) + (K(b38) + K(b39)) * CC(1);
        /* ch4 */
        PR(2) = 0.e0;
        PE(2) = K(c2) * CC(2) + K(c1a) * CC(1) + K(c1b) * CC(1) + K(c1c) * CC(1) + K(d5) * CC(3);
        /* h2o */
        PR(3) = K(c2) * CC(2) * CK(2) + K(c8) * CC(2) * CK(28) + K(c17a) * CK(30) * CC(2) + K(c17b) * CK(30) * CC(2) +
                (K(a17) * CC(2) + a23c * CC(14)) * CC(6) + K(a19) * CC(2) * h2 + K(a30) * CC(2) * CK(17) +
                K(a31) * CC(2) * CC(2) + K(b27) * CC(2) * CK(5) * parthno3 + K(d11) * CC(2) * CK(13) * parthcl;
        PE(3) = (TJ(h2o) + K(a1et) * CC(1)) * parth2o;
        /* noy */
        PR(4) = 2. * K(b39) * CC(1) * CK(1);
        PE(4) = 2. * K(b6) * CC(10) * CC(8) + rain_hno3 * CK(5) + rain_hno4 * CK(22);
        PE(4) = PE(4) / CK(4);
        /* hno3 */
        PR(5) = K(b22) * CC(2) * CC(7) + HET(1) * CK(14) * CK(3) + HET(2) * CK(14) * CK(13) +
                2. * HET(3) * CK(6) * CK(3) + HET(4) * CK(6) * CK(13) + HET(6) * CK(20) * CK(3);
        PE(5) = (TJ(hno3) + K(b27) * CC(2)) * parthno3 + rain_hno3;
        /* n2o5 */
        PR(6) = K(b12) * CC(13) * CC(7);
        PE(6) = TJ(n2o5) + K(b32) * hnm + HET(3) * CK(3) + HET(4) * CK(13);
        /* cly */
        PR(7) = 3. * (TJ(cfc11) + K(d90) * CC(1)) * CK(31) + 2. * (TJ(cfc12) + K(d91) * CC(1)) * CK(32) +
                3. * (TJ(cfc113) + K(d92) * CC(1)) * CK(33) + 4. * (TJ(ccl4) + K(d93) * CC(1)) * CK(34) +
                3. * (TJ(ch3ccl3) + K(d94) * CC(2)) * CK(35) + 1. * (TJ(ch3cl) + K(d95) * CC(2)) * CK(36) +
                1. * (TJ(hcfc22) + K(d96) * CC(1) + K(d97) * CC(2)) * CK(37) +
                1. * (TJ(h1211) + K(e52) * CC(1)) * CK(39);
        PE(7) = rain_hcl * CK(13);
        PE(7) = PE(7) / CK(7);
        /* ox */
        double ratio = TJ(cl2o2) / (TJ(cl2o2) + K(d61) * hnm);
        PR(8) = 2. * TJ(o2) * o2 + K(a26) * CC(6) * CC(8) + K(c5) * CC(8) * CK(29);
        t01 = 2. * K(hk1) * CC(4) * CC(4);
        t02 = 2. * K(hk3) * CC(5) * CC(4);
        t03 = 2. * K(b3) * CC(7) * CC(4);
        t04 = 2. * K(d3) * CC(11) * CC(4);
        t05 = 2. * K(d60) * ratio * CC(11) * CC(11);
        t06 = fmin(TJ(hocl) * CK(15), K(d33) * CC(6) * CC(11));
        t07 = 2. * fmin(K(e5c) * CC(12) * CC(11), TJ(brcl) * CK(27));
        t08 = 2. * K(e5b) * CC(12) * CC(11) * day;
        t09 = fmin(K(e15) * CC(12) * CC(6), TJ(hobr) * CK(26));
        t10 = 2. * K(e6) * CC(12) * CC(12) * day;
        t11 = 2. * (TJ(no3_no) / fmax(TJ(no3_no) + TJ(no3_no2), 1.e-30)) * TJ(clono2_cl) * CK(14);
        t12 = (K(a2) * CC(14) + K(a6) * CC(2) + K(a6b) * CC(6)) * CC(5) + (K(a5) * CC(2) + K(a7) * CC(6)) * CC(4);
        t13 = 2. * K(b9) * CC(7) * CC(5) * TJ(no3_no) / fmax(TJ(no3_no) + TJ(no3_no2), 1.e-30);
        PE(8) = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13;
        PE(8) = PE(8) / CK(8);
        /* co */
        PR(9) = TJ(co2) * co2 + TJ(ch2o_co) * CK(28) + K(c12) * hco * o2;
        PE(9) = K(a36) * CC(2);
        /* oclo */
        PR(10) = K(e5a) * CC(12) * CC(11);
        PE(10) = TJ(oclo);
        /* ox passif, h2so4 */
        PR(11) = 0.;
        PE(11) = 0.;
        PR(12) = 0.;
        PE(12) = 0.;
        /* hcl */
        PR(13) = (K(c10) * CK(28) + K(d5) * CK(2) + K(d7) * CC(6) + K(d6) * h2) * CC(3) + K(d9) * CC(2) * CC(11);
        PE(13) = (TJ(hcl) + K(d11) * CC(2)) * parthcl + HET(2) * CK(14) + HET(4) * CK(6) + HET(5) * CK(15) +
                 HET(7) * CK(26) + rain_hcl;
        /* clono2 */
        PR(14) = K(d31) * CC(7) * CC(11);
        PE(14) = TJ(clono2_cl) + TJ(clono2_clo) + K(d32) * CC(4) + HET(1) * CK(3) + HET(2) * CK(13);
        /* hocl */
        PR(15) = K(d33) * CC(6) * CC(11) + HET(1) * CK(14) * CK(3);
        PE(15) = TJ(hocl) + K(d34) * CC(2) + K(d35) * CC(4) + K(d37) * CC(3) + HET(5) * CK(13) + HET(9) * CK(19);
        /* cl2 */
        PR(16) = K(d37) * CK(15) * CC(3) + K(d62) * CC(11) * CC(11) + HET(2) * CK(14) * CK(13) +
                 HET(5) * CK(15) * CK(13);
        PE(16) = TJ(cl2);
        /* h2o2 */
        PR(17) = K(a27) * CC(6) * CC(6);
        PE(17) = TJ(h2o2) + K(a30) * CC(2) + rain_h2o2;
        /* clno2 */
        PR(18) = K(d36) * CC(3) * CC(7) + HET(4) * CK(6) * CK(13);
        PE(18) = TJ(clno2);
        /* hbr */
        PR(19) = K(e7) * CC(6) * CC(9) + K(c19) * CK(28) * CC(9);
        PE(19) = (K(e11) * CC(2) + K(e9) * CC(1) + TJ(hbr)) * parthbr + HET(8) * CK(26) + HET(9) * CK(15) + rain_hbr;
        /* brono2 */
        PR(20) = K(e13) * CC(12) * CC(7);
        PE(20) = TJ(brono2) + K(e8) * CC(4) + HET(6) * CK(3);
        /* nox */
        PR(21) = (TJ(hno4) + K(b28) * CC(2) + K(b24) * hnm) * CK(22) + TJ(hno3) * CK(5) * parthno3 +
                 2. * (TJ(n2o5) + K(b32) * hnm) * CK(6) + 2. * K(b39) * CC(1) * CK(1) + TJ(clno2) * CK(18) +
                 K(b27) * CK(5) * parthno3 * CC(2) + K(d32) * CK(14) * CC(4) +
                 (TJ(clono2_cl) + TJ(clono2_clo)) * CK(14) + TJ(brono2) * CK(20) + K(e8) * CK(20) * CC(4);
        PE(21) = (K(d31) * CC(11) + K(b22) * CC(2) + K(b23) * CC(6) + 2. * K(b12) * CC(13) + K(d36) * CC(3) +
                  K(e13) * CC(12)) *
                     CC(7) +
                 2. * K(b6) * CC(10) * CC(8);
        PE(21) = PE(21) / CK(21);
        /* ho2no2 */
        PR(22) = K(b23) * CC(6) * CC(7);
        PE(22) = TJ(hno4) + K(b28) * CC(2) + K(b24) * hnm + rain_hno4;
        /* clox */
        t01 = 2. * (K(d61) * hnm + TJ(cl2o2)) * CK(25);
        t02 = (TJ(clono2_cl) + TJ(clono2_clo) + K(d32) * CC(4)) * CK(14);
        t03 = (TJ(hocl) + K(d34) * CC(2) + K(d35) * CC(4)) * CK(15);
        t04 = TJ(oclo) * CK(10) + (TJ(hcl) + K(d11) * CC(2)) * CK(13) * parthcl;
        t05 = 2. * TJ(cl2) * CK(16);
        t06 = TJ(clno2) * CK(18);
        t07 = TJ(brcl) * CK(27);
        t08 = 3. * (TJ(cfc11) + K(d90) * CC(1)) * CK(31);
        t09 = 2. * (TJ(cfc12) + K(d91) * CC(1)) * CK(32);
        t10 = 3. * (TJ(cfc113) + K(d92) * CC(1)) * CK(33);
        t11 = 4. * (TJ(ccl4) + K(d93) * CC(1)) * CK(34);
        t12 = 3. * (TJ(ch3ccl3) + K(d94) * CC(2)) * CK(35);
        t13 = 1. * (TJ(ch3cl) + K(d95) * CC(2)) * CK(36);
        t14 = 1. * (TJ(hcfc22) + K(d96) * CC(1) + K(d97) * CC(2)) * CK(37);
        PR(23) = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13 + t14;
        PE(23) = (K(d31) * CC(7) + 2. * K(d60) * CC(11) + 2. * K(d62) * CC(11) + K(e5a) * CC(12) + K(e5c) * CC(12) +
                  K(d9) * CC(2) + K(d33) * CC(6)) *
                     CC(11) +
                 (K(c10) * CK(28) + K(d5) * CK(2) + K(d7) * CC(6) + K(d6) * h2 + K(d36) * CC(7) + K(d37) * CK(15)) *
                     CC(3);
        PE(23) = PE(23) / CK(23);
        /* brox */
        PR(24) = TJ(hobr) * CK(26) + TJ(brono2) * CK(20) + K(e8) * CK(20) * CC(4) + K(e16) * CK(26) * CC(4) +
                 TJ(brcl) * CK(27) + (K(e11) * CC(2) + K(e9) * CC(1) + TJ(hbr)) * CK(19) * parthbr +
                 2. * HET(8) * CK(19) * CK(26);
        PE(24) = (K(e13) * CC(7) + K(e5c) * CC(11) + K(e15) * CC(6)) * CC(12) + K(c19) * CC(9) * CK(28) +
                 K(e7) * CC(9) * CC(6);
        PE(24) = PE(24) / CK(24);
        /* cl2o2 */
        PR(25) = K(d60) * CC(11) * CC(11);
        PE(25) = TJ(cl2o2) + K(d61) * hnm;
        /* hobr */
        PR(26) = K(e15) * CC(12) * CC(6) + HET(6) * CK(20) * CK(3);
        PE(26) = TJ(hobr) + K(e16) * CC(4) + HET(7) * CK(13) + HET(8) * CK(19);
        /* brcl */
        PR(27) = K(e5c) * CC(11) * CC(12) + HET(7) * CK(26) * CK(13) + HET(9) * CK(19) * CK(15);
        PE(27) = TJ(brcl);
        /* ch2o */
        PR(28) = (K(c1c) * CC(1) * CK(2) + K(c3) * CC(4) * CC(15) + K(c15) * ch3o * o2 + K(c17b) * CC(2) * CK(30));
        PE(28) = K(c8) * CC(2) + K(c9) * CC(4) + K(c10) * CC(3) + K(c19) * CC(9) + TJ(ch2o_hco) + TJ(ch2o_co) +
                 rain_ch2o;
        /* ch3o2 */
        PR(29) = K(c4) * CC(15) * o2 + K(c17a) * CC(2) * CK(30);
        PE(29) = 2. * K(c14) * CK(29) + K(c7) * CC(6) + K(c5) * CC(8) + K(c18) * CC(11);
        /* ch3o2h */
        PR(30) = K(c7) * CK(29) * CC(6);
        PE(30) = K(c17a) * CC(2) + K(c17b) * CC(2) + TJ(ch3o2h) + rain_ch3o2h;
        /* source gases */
        PR(31) = 0.;
        PE(31) = TJ(cfc11) + K(d90) * CC(1);
        PR(32) = 0.;
        PE(32) = TJ(cfc12) + K(d91) * CC(1);
        PR(33) = 0.;
        PE(33) = TJ(cfc113) + K(d92) * CC(1);
        PR(34) = 0.;
        PE(34) = TJ(ccl4) + K(d93) * CC(1);
        PR(35) = 0.;
        PE(35) = TJ(ch3ccl3) + K(d94) * CC(2);
        PR(36) = 0.;
        PE(36) = TJ(ch3cl) + K(d95) * CC(2);
        PR(37) = 0.;
        PE(37) = TJ(hcfc22) + K(d96) * CC(1) + K(d97) * CC(2);
        PR(38) = 0.;
        PE(38) = TJ(ch3br) + K(e50) * CC(1) + K(e51) * CC(2);
        PR(39) = 0.;
        PE(39) = TJ(h1211) + K(e52) * CC(1);
        PR(40) = 0.;
        PE(40) = TJ(h1301) + K(e53) * CC(1);
        /* bry */
        PR(41) = (TJ(ch3br) + K(e50) * CC(1) + K(e51) * CC(2)) * CK(38) + (TJ(h1211) + K(e52) * CC(1)) * CK(39) +
                 (TJ(h1301) + K(e53) * CC(1)) * CK(40) + 2. * (K(e54) * CC(2) + TJ(ch2br2)) * CK(42);
        PE(41) = rain_hbr * CK(19);
        PE(41) = PE(41) / CK(41);
        /* ch2br2 */
        PR(42) = 0.;
        PE(42) = TJ(ch2br2) + K(e54) * CC(2);
        /* hno3 gas */
        PR(NBCON) = 0.;
        PE(NBCON) = 0.;
    }
    /* ---- semi-implicit update, F:2364-2372 ---- */
    for (int m = 1; m <= NBCON - 1; m++)
        for (size_t c = 0; c < n; c++) CK(m) = (w->ck0[(size_t)(m - 1) * n + c] + dt * PR(m)) / (1. + dt * PE(m));
#undef PR
#undef PE
#undef K
#undef CK
#undef CC
#undef TJ
#undef HET
}

/* ============================================================================
 * Oracle-C: the fixed point of one pass of the iteration (F:1350-2372),
 * G(x) = x with x = (ck(1..42), cc(1..15)), by Newton's method on
 * F(x) = G(x) - x. The Jacobian of G is taken by forward differences of the
 * pass itself (cells are independent within a pass, so all cells of a
 * workspace are perturbed at once), each cell's 57x57 system is solved by LU
 * with partial pivoting. Converged when |G(x) - x| is below tol relative to
 * max(|x|, 1e-40*hnm) for every unknown (the night NO2 fixed point sits near
 * 1e-30 molecules/cm3, inside the max(NO2, 1e-30) of F:1722, and NO3
 * depends on which side of that clamp NO2 is).
 *
 * Newton from the reference's 5-pass state does not converge in every cell:
 * where the pass map oscillates (warm cells at high pressure, some polar
 * night cells) that state can lie outside Newton's basin. A cell that has not
 * converged moves on to the next start of a fixed sequence, and the first
 * start whose iteration converges gives its answer:
 *   stage 1  Newton from the 5-pass state (the reference's own answer);
 *   stage 2  Newton from the step's initial state (no pass);
 *   stage 3-5  Newton from the 1-, 2- and 3-pass states;
 *   stage 6  pseudo-transient continuation from the 5-pass state:
 *            (I/d - F'(x)) dx = F(x), d grown by the ratio of successive
 *            residuals (switched evolution relaxation), i.e. relaxed passes
 *            that turn into Newton steps as the residual falls.
 * Newton steps are halved while they raise the residual (up to 8 times);
 * a continuation step is shortened as a whole so that no component falls
 * below a tenth of its value (stepping component by component towards zero
 * finds spurious roots with Br radicals near 1e-120); in every stage a
 * component still driven negative is set to a tenth of its previous value.
 * Some night cells have two fixed points (NO2 on either side of the clamp);
 * the sequence takes the one reached from the state nearest the reference's
 * passes first. Each stage works on a compacted copy of the cells still
 * iterating, so converged cells cost nothing.
 * ========================================================================== */
#define NX (NBCON - 1 + NCM)

static void get_x(const work* w, size_t c, double* x) {
    for (int m = 0; m < NBCON - 1; m++) x[m] = w->ck[c + w->n * m];
    for (int m = 0; m < NCM; m++) x[NBCON - 1 + m] = w->cc[c + w->n * m];
}
static void put_x(work* w, size_t c, const double* x) {
    for (int m = 0; m < NBCON - 1; m++) w->ck[c + w->n * m] = x[m];
    for (int m = 0; m < NCM; m++) w->cc[c + w->n * m] = x[NBCON - 1 + m];
}

/* G for every cell of the workspace at the states X (n x NX), into GX */
static void block_map(const orc_grid* g, double dt, work* w, const double* X, double* GX) {
    for (size_t c = 0; c < w->n; c++) put_x(w, c, X + c * NX);
    orc_pass(g, dt, w);
    for (size_t c = 0; c < w->n; c++) get_x(w, c, GX + c * NX);
}

static int lu_solve(double* A, double* b, int n) {
    /* A row-major n x n, overwritten; b overwritten with the solution */
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = fabs(A[k * n + k]);
        for (int i = k + 1; i < n; i++)
            if (fabs(A[i * n + k]) > best) best = fabs(A[i * n + k]), p = i;
        if (!(best > 0.)) return -1;
        if (p != k) {
            for (int j = 0; j < n; j++) {
                double t = A[k * n + j];
                A[k * n + j] = A[p * n + j];
                A[p * n + j] = t;
            }
            double t = b[k];
            b[k] = b[p];
            b[p] = t;
        }
        for (int i = k + 1; i < n; i++) {
            double f = A[i * n + k] / A[k * n + k];
            if (f == 0.) continue;
            for (int j = k; j < n; j++) A[i * n + j] -= f * A[k * n + j];
            b[i] -= f * b[k];
        }
    }
    for (int k = n - 1; k >= 0; k--) {
        double s = b[k];
        for (int j = k + 1; j < n; j++) s -= A[k * n + j] * b[j];
        b[k] = s / A[k * n + k];
    }
    return 0;
}

static const double g_floor = 1e-40;
/* max_i |G(x)_i - x_i| / max(|x_i|, fl); NaN gives NaN (never converged) */
static double fnorm(const double* x, const double* gx, double fl) {
    double m = 0.;
    for (int i = 0; i < NX; i++) {
        double s = fmax(fabs(x[i]), fl);
        double r = fabs(gx[i] - x[i]) / s;
        if (!(r <= m)) m = r;
    }
    return m;
}

enum { STAGE_NEWTON = 0, STAGE_PTC = 1 };

/* One stage over the cells act[0..na) of the block workspace w, each
 * starting from its row of Xb (n x NX, in/out). A converged cell gets
 * conv = stage_id, its iterate in Xb, its Newton steps added to iters and its
 * residual in res. Returns the cells still unconverged, left in act. */
static size_t newton_stage(const orc_grid* g, double dt, const work* w, size_t* act, size_t na, double* Xb,
                           int mode, int stage_id, int maxit, int* iters, double* res, int* conv) {
    if (!na) return 0;
    work* ws = work_subset(w, act, na);
    size_t m = na;
    size_t* loc = (size_t*)malloc(sizeof(size_t) * na);  /* block index of each workspace cell */
    size_t* keep = (size_t*)malloc(sizeof(size_t) * na);
    double* X = (double*)malloc(sizeof(double) * na * NX);
    double* GX = (double*)malloc(sizeof(double) * na * NX);
    double* XP = (double*)malloc(sizeof(double) * na * NX);
    double* GP = (double*)malloc(sizeof(double) * na * NX);
    double* J = (double*)malloc(sizeof(double) * na * NX * NX);
    double* H = (double*)malloc(sizeof(double) * na);
    double* D = (double*)malloc(sizeof(double) * na);  /* PTC pseudo time step */
    double* F0 = (double*)malloc(sizeof(double) * na); /* residual at X */
    int* dead = (int*)calloc(na, sizeof(int));
    for (size_t c = 0; c < na; c++) {
        loc[c] = act[c];
        memcpy(X + c * NX, Xb + act[c] * NX, sizeof(double) * NX);
        D[c] = 0.5;
    }
    block_map(g, dt, ws, X, GX);
    size_t left = 0;
    for (int it = 0;; it++) {
        /* convergence test; keep the cells still iterating */
        size_t k = 0;
        for (size_t c = 0; c < m; c++) {
            const double f = fnorm(X + c * NX, GX + c * NX, g_floor * ws->hnm[c]);
            const size_t b = loc[c];
            if (f < g->tol) {
                conv[b] = stage_id;
                iters[b] += it;
                res[b] = f;
                memcpy(Xb + b * NX, X + c * NX, sizeof(double) * NX);
                continue;
            }
            if (it == maxit || dead[c]) {
                res[b] = f;
                iters[b] += it;
                act[left++] = b;
                continue;
            }
            F0[k] = f;
            keep[k] = c;
            if (k != c) {
                memcpy(X + k * NX, X + c * NX, sizeof(double) * NX);
                memcpy(GX + k * NX, GX + c * NX, sizeof(double) * NX);
                D[k] = D[c];
                loc[k] = loc[c];
                dead[k] = 0;
            }
            k++;
        }
        if (k == 0) break;
        if (k < m) {
            work* w2 = work_subset(ws, keep, k);
            work_free(ws);
            ws = w2;
            m = k;
        }
        /* forward-difference Jacobian of G, column j for all cells at once */
        for (int j = 0; j < NX; j++) {
            memcpy(XP, X, sizeof(double) * m * NX);
            for (size_t c = 0; c < m; c++) {
                const double xj = X[c * NX + j];
                const double h = 1e-7 * fmax(fabs(xj), g_floor * 1e5 * ws->hnm[c]);
                H[c] = h;
                XP[c * NX + j] = xj + h;
            }
            block_map(g, dt, ws, XP, GP);
            for (size_t c = 0; c < m; c++)
                for (int i = 0; i < NX; i++)
                    J[(c * NX + i) * NX + j] = (GP[c * NX + i] - GX[c * NX + i]) / H[c];
        }
        /* the step: Newton (J_G - I) dx = -(G - x); PTC (I/d - (J_G - I)) dx = G - x */
        for (size_t c = 0; c < m; c++) {
            double* A = J + c * NX * NX;
            double bb[NX];
            for (int i = 0; i < NX; i++) {
                const double fi = GX[c * NX + i] - X[c * NX + i];
                if (mode == STAGE_PTC) {
                    for (int q = 0; q < NX; q++) A[i * NX + q] = -A[i * NX + q];
                    A[i * NX + i] += 1. + 1. / D[c];
                    bb[i] = fi;
                } else {
                    A[i * NX + i] -= 1.;
                    bb[i] = -fi;
                }
            }
            memcpy(XP + c * NX, X + c * NX, sizeof(double) * NX); /* the previous iterate */
            if (lu_solve(A, bb, NX) != 0) {
                dead[c] = 1;
                continue;
            }
            double lam = 1.;
            if (mode == STAGE_PTC) /* the whole step shortened: no component below a tenth */
                for (int i = 0; i < NX; i++) {
                    const double x0 = X[c * NX + i];
                    if (x0 > 0. && x0 + bb[i] < 0.1 * x0) lam = fmin(lam, -0.9 * x0 / bb[i]);
                }
            for (int i = 0; i < NX; i++) {
                const double x0 = X[c * NX + i];
                const double xn = x0 + lam * bb[i];
                X[c * NX + i] = xn < 0. ? x0 / 10. : xn;
            }
        }
        block_map(g, dt, ws, X, GP);
        if (mode == STAGE_PTC) {
            for (size_t c = 0; c < m; c++) {
                const double fn_new = fnorm(X + c * NX, GP + c * NX, g_floor * ws->hnm[c]);
                double r = fn_new > 0. ? F0[c] / fn_new : 1e10;
                if (!(r <= 1e10)) r = 1e10;
                D[c] = fmin(fmax(D[c] * r, 1e-3), 1e12);
            }
        } else {
            /* halve steps that raise the residual */
            for (int half = 0; half < 8; half++) {
                int any = 0;
                for (size_t c = 0; c < m; c++) {
                    if (dead[c]) continue;
                    const double fn_new = fnorm(X + c * NX, GP + c * NX, g_floor * ws->hnm[c]);
                    if (!(fn_new <= F0[c]) && fn_new > g->tol) {
                        for (int i = 0; i < NX; i++) X[c * NX + i] = 0.5 * (X[c * NX + i] + XP[c * NX + i]);
                        any = 1;
                    }
                }
                if (!any) break;
                block_map(g, dt, ws, X, GP);
            }
        }
        memcpy(GX, GP, sizeof(double) * m * NX);
    }
    work_free(ws);
    free(loc); free(keep); free(X); free(GX); free(XP); free(GP); free(J); free(H); free(D); free(F0);
    free(dead);
    return left;
}

/* Oracle-C over one block: X0 holds every cell's state before the passes
 * (n x NX); w holds the 5-pass state. With X0 NULL (a given start state in
 * w) only stage 1 runs: Newton from that state, to the fixed point nearest
 * it. On return w holds each converged cell's fixed point and each
 * unconverged cell's start state. Per cell:
 * iters = Newton steps over all stages (-steps-1 if not converged),
 * res = the final residual, stage = the stage that converged (0: none). */
static void orc_newton_block(const orc_grid* g, double dt, work* w, const double* X0, int* iters, double* res,
                             int* stage) {
    const size_t n = w->n;
    double* X5 = (double*)malloc(sizeof(double) * n * NX);
    double* Xb = (double*)malloc(sizeof(double) * n * NX);
    size_t* act = (size_t*)malloc(sizeof(size_t) * n);
    for (size_t c = 0; c < n; c++) {
        get_x(w, c, X5 + c * NX);
        act[c] = c;
        iters[c] = 0;
        stage[c] = 0;
    }
    memcpy(Xb, X5, sizeof(double) * n * NX);
    const int maxit = g->maxiter > 0 ? g->maxiter : 60;
    size_t na = newton_stage(g, dt, w, act, n, Xb, STAGE_NEWTON, 1, maxit, iters, res, stage);
    for (int np = 0; np <= 3 && na && X0; np++) {
        /* restart from the np-pass state */
        work* ws = work_subset(w, act, na);
        for (size_t c = 0; c < na; c++) put_x(ws, c, X0 + act[c] * NX);
        for (int p = 0; p < np; p++) orc_pass(g, dt, ws);
        for (size_t c = 0; c < na; c++) get_x(ws, c, Xb + act[c] * NX);
        work_free(ws);
        na = newton_stage(g, dt, w, act, na, Xb, STAGE_NEWTON, 2 + np, 40, iters, res, stage);
    }
    if (na && X0) {
        for (size_t c = 0; c < na; c++) memcpy(Xb + act[c] * NX, X5 + act[c] * NX, sizeof(double) * NX);
        na = newton_stage(g, dt, w, act, na, Xb, STAGE_PTC, 6, 4 * maxit, iters, res, stage);
    }
    for (size_t c = 0; c < n; c++) {
        if (stage[c] == 0) {
            iters[c] = -iters[c] - 1;
            put_x(w, c, X5 + c * NX);
        } else {
            put_x(w, c, Xb + c * NX);
        }
    }
    free(X5); free(Xb); free(act);
}

/* ============================================================================
 * chem3d, F:601-2412 — one block of nl longitudes of row ilat
 * ========================================================================== */
static int orc_chem3d_block(const orc_grid* g, work* w, int ilat, int i0, double daynum, double dt,
                            const double* alt, const double* trajlon, const double* trajlat,
                            const double* trajpre, const double* trajtem, int irapp, double* qj1, double* hc,
                            double* vsed3d, double* parth2osed, double* parthno3sed, double* surfarea,
                            double* sza3d, double* diag) {
    const int nl = w->nl, nb = w->nb;
    const size_t n = w->n;
    /* ---- air density and fixed gases, F:800-812 ---- */
    for (int k = 0; k < nb; k++)
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            w->t[c] = GT(trajtem, i0 + i, ilat, k, irapp);
            w->pm[c] = GT(trajpre, i0 + i, ilat, k, irapp);
            w->hnm[c] = GT(trajpre, i0 + i, ilat, k, irapp) / (GT(trajtem, i0 + i, ilat, k, irapp) * 1.38e-19);
            w->n2[c] = 0.78 * w->hnm[c];
            w->o2[c] = 0.21 * w->hnm[c];
            w->co2[c] = 360.e-6 * w->hnm[c];
            w->h2[c] = 5.e-7 * w->hnm[c];
        }
    /* ---- number densities, F:818-833 ---- */
    for (int m = 0; m < NBCON; m++)
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) {
                const size_t c = R(i, k);
                w->ck0[c + n * m] = G4(qj1, i0 + i, ilat, k, m) * w->hnm[c];
                w->ck[c + n * m] = w->ck0[c + n * m];
            }
    for (int m = 0; m < NCM; m++)
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) {
                const size_t c = R(i, k);
                w->cc[c + n * m] = G4(hc, i0 + i, ilat, k, m) * w->hnm[c];
            }
    /* ---- total, zenith, F:839-851 ---- */
    orc_total(g, trajpre, irapp, ilat, i0, hc, w);
    orc_zenith(g, trajlon, trajlat, irapp, ilat, i0, daynum, w);
    for (int k = 0; k < nb; k++)
        for (int i = 0; i < nl; i++) GB(sza3d, i0 + i, ilat, k) = w->sza[R(i, k)];
    /* ---- phot, F:857 ---- */
    orc_phot(g, ilat, i0, alt, w);
    /* ---- het init, F:864-880 ---- */
    for (size_t c = 0; c < n; c++) {
        for (int m = 0; m < 9; m++) w->het[c + n * m] = 0.;
        w->parth2o[c] = 1.;
        w->parthno3[c] = 1.;
        w->parthcl[c] = 1.;
        w->parthbr[c] = 1.;
        w->surf[c] = 0.;
    }
    /* ---- analytic, F:898-912 ---- */
    orc_analytic(g, ilat, i0, surfarea, w);
    for (int k = 0; k < nb; k++)
        for (int i = 0; i < nl; i++) {
            const size_t c = R(i, k);
            GB(vsed3d, i0 + i, ilat, k) = w->vsed[c];
            GB(parth2osed, i0 + i, ilat, k) = w->parth2o[c];
            GB(parthno3sed, i0 + i, ilat, k) = w->parthno3sl[c];
        }
    /* ---- rate constants, F:920-1306 ---- */
    orc_rates(g, w);
    /* ---- rainout, F:1315-1338 ---- */
    {
        const double rain_h2o = 100.e-6, rain_rate = 1.e-6;
        for (size_t c = 0; c < n; c++) {
            if (w->ck[c + n * 2] / w->hnm[c] >= rain_h2o) {
                w->rain_hno3[c] = rain_rate;
                w->rain_hno4[c] = 0.;
                w->rain_hcl[c] = rain_rate;
                w->rain_hbr[c] = rain_rate;
                w->rain_h2o2[c] = rain_rate;
                w->rain_ch2o[c] = 0.;
                w->rain_ch3o2h[c] = 0.;
            } else {
                w->rain_hno3[c] = 0.;
                w->rain_hno4[c] = 0.;
                w->rain_hcl[c] = 0.;
                w->rain_hbr[c] = 0.;
                w->rain_h2o2[c] = 0.;
                w->rain_ch2o[c] = 0.;
                w->rain_ch3o2h[c] = 0.;
            }
        }
    }
    /* ---- diagnostics of the rate stage ---- */
    if (diag) {
        const size_t ncd = (size_t)g->nlon * g->nlat * g->nivbas;
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) {
                const size_t c = R(i, k);
                const size_t cell = (size_t)(i0 + i) + (size_t)g->nlon * ((size_t)ilat + (size_t)g->nlat * k);
#define DG(d) diag[(size_t)(d)*ncd + cell]
                DG(REPROBUS_DIAG_HNM) = w->hnm[c];
                DG(REPROBUS_DIAG_SZA) = w->sza[c];
                DG(REPROBUS_DIAG_O3T) = w->o3t[c];
                for (int m = 0; m < NPHOT; m++) DG(REPROBUS_DIAG_TJ + m) = w->tj[c + n * m];
                for (int m = 0; m < 9; m++) DG(REPROBUS_DIAG_HET + m) = w->het[c + n * m];
                DG(REPROBUS_DIAG_PARTHNO3) = w->parthno3[c];
                DG(REPROBUS_DIAG_PARTHNO3SL) = w->parthno3sl[c];
                DG(REPROBUS_DIAG_PARTH2O) = w->parth2o[c];
                DG(REPROBUS_DIAG_PARTHCL) = w->parthcl[c];
                DG(REPROBUS_DIAG_VSED) = w->vsed[c];
                DG(REPROBUS_DIAG_SURFAREA) = w->surf[c];
                for (int m = 0; m < K_COUNT; m++) DG(REPROBUS_DIAG_RATE + m) = w->rk[c + n * m];
#undef DG
            }
    }
    /* ---- given state x: one pass from it (map residual), or Newton from it ---- */
    const int given = g->x_qj1 && g->x_hc;
    if (given) {
        for (int m = 0; m < NBCON - 1; m++)
            for (int k = 0; k < nb; k++)
                for (int i = 0; i < nl; i++) w->ck[R(i, k) + n * m] = G4(g->x_qj1, i0 + i, ilat, k, m) * w->hnm[R(i, k)];
        for (int m = 0; m < NCM; m++)
            for (int k = 0; k < nb; k++)
                for (int i = 0; i < nl; i++) w->cc[R(i, k) + n * m] = G4(g->x_hc, i0 + i, ilat, k, m) * w->hnm[R(i, k)];
    }
    if (given && !g->newton) {
        double* X0 = (double*)malloc(sizeof(double) * n * NX);
        for (size_t c = 0; c < n; c++) get_x(w, c, X0 + c * NX);
        orc_pass(g, dt, w);
        for (size_t c = 0; c < n; c++) {
            double gx[NX];
            get_x(w, c, gx);
            if (g->cellres) {
                const size_t cell = (size_t)(i0 + c % nl) + (size_t)g->nlon * ((size_t)ilat + (size_t)g->nlat * (c / nl));
                g->cellres[cell] = fnorm(X0 + c * NX, gx, 1e-20 * w->hnm[c]);
            }
        }
        free(X0);
    }
    /* ---- iteration, F:1348-2378 ---- */
    double* Xstart = NULL; /* Oracle-C restarts from the state before the passes */
    if (g->newton && !given) {
        Xstart = (double*)malloc(sizeof(double) * n * NX);
        for (size_t c = 0; c < n; c++) get_x(w, c, Xstart + c * NX);
    }
    int passes = 0;
    if (given) {
        passes = g->newton ? 0 : 1;
    } else if (g->niter > 0) {
        for (int it = 0; it < g->niter; it++) orc_pass(g, dt, w);
        passes = g->niter;
    } else {
        /* iterate the same map to its fixed point */
        for (int it = 0; it < g->maxiter; it++) {
            memcpy(w->cc_prev, w->cc, sizeof(double) * n * NCM);
            memcpy(w->ck_prev, w->ck, sizeof(double) * n * NBCON);
            orc_pass(g, dt, w);
            passes++;
            double dmax = 0.;
            for (size_t q = 0; q < n * NCM; q++) {
                double a = w->cc[q], b = w->cc_prev[q];
                double s = fmax(fabs(a), fabs(b));
                if (s > 0.) dmax = fmax(dmax, fabs(a - b) / s);
            }
            for (size_t q = 0; q < n * (NBCON - 1); q++) {
                double a = w->ck[q], b = w->ck_prev[q];
                double s = fmax(fabs(a), fabs(b));
                if (s > 0.) dmax = fmax(dmax, fabs(a - b) / s);
            }
            if (dmax < g->tol) break;
        }
    }
    if (g->newton) {
        /* Oracle-C: from the passes' result (or from the given state),
         * Newton to the fixed point */
        int* it = (int*)malloc(sizeof(int) * n);
        int* stg = (int*)malloc(sizeof(int) * n);
        double* res = (double*)malloc(sizeof(double) * n);
        orc_newton_block(g, dt, w, Xstart, it, res, stg);
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) {
                const size_t cell = (size_t)(i0 + i) + (size_t)g->nlon * ((size_t)ilat + (size_t)g->nlat * k);
                if (g->cellstat) g->cellstat[cell] = it[R(i, k)];
                if (g->cellres) g->cellres[cell] = res[R(i, k)];
                if (g->cellstage) g->cellstage[cell] = stg[R(i, k)];
            }
        free(it);
        free(stg);
        free(res);
    }
    free(Xstart);
    /* ---- write-back, F:2380-2410 ---- */
    for (int m = 0; m < NBCON - 1; m++)
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) G4(qj1, i0 + i, ilat, k, m) = w->ck[R(i, k) + n * m] / w->hnm[R(i, k)];
    for (int k = 0; k < nb; k++)
        for (int i = 0; i < nl; i++)
            G4(qj1, i0 + i, ilat, k, NBCON - 1) = w->ck[R(i, k) + n * 4] * w->parthno3[R(i, k)] / w->hnm[R(i, k)];
    for (int m = 0; m < NCM; m++)
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nl; i++) G4(hc, i0 + i, ilat, k, m) = w->cc[R(i, k) + n * m] / w->hnm[R(i, k)];
    return passes;
}

#define ORC_BLOCK 4

void orc_chem3d(const orc_grid* g, int ilat, double daynum, double dt, const double* alt, const double* trajlon,
                const double* trajlat, const double* trajpre, const double* trajtem, int irapp, double* qj1,
                double* hc, double* vsed3d, double* parth2osed, double* parthno3sed, double* surfarea,
                double* sza3d, double* diag, int* passes) {
    int pmax = 0;
    for (int i0 = 0; i0 < g->nlon; i0 += ORC_BLOCK) {
        int nl = g->nlon - i0 < ORC_BLOCK ? g->nlon - i0 : ORC_BLOCK;
        work* w = work_alloc(nl, g->nivbas);
        int p = orc_chem3d_block(g, w, ilat, i0, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc,
                                 vsed3d, parth2osed, parthno3sed, surfarea, sza3d, diag);
        if (p > pmax) pmax = p;
        work_free(w);
    }
    if (passes) *passes = pmax;
}

/* ============================================================================
 * conserv, F:2526-2616
 * ========================================================================== */
void orc_conserv(const orc_grid* g, int ilat0, int ilat1, double* qj1, double* hc) {
    for (int k = 0; k < g->nivbas; k++)
        for (int j = ilat0; j <= ilat1; j++)
            for (int i = 0; i < g->nlon; i++) {
#define Q(m) G4(qj1, i, j, k, (m)-1)
#define H(m) G4(hc, i, j, k, (m)-1)
                double totmas = Q(10) + Q(13) + Q(14) + Q(15) + 2. * Q(16) + Q(18) + Q(23) + 2. * Q(25);
                double rapcly = (Q(7) - Q(27)) / totmas;
                H(3) = H(3) * rapcly;
                H(11) = H(11) * rapcly;
                Q(10) = Q(10) * rapcly;
                Q(13) = Q(13) * rapcly;
                Q(14) = Q(14) * rapcly;
                Q(15) = Q(15) * rapcly;
                Q(16) = Q(16) * rapcly;
                Q(18) = Q(18) * rapcly;
                Q(23) = Q(23) * rapcly;
                Q(25) = Q(25) * rapcly;
                totmas = Q(5) + 2. * Q(6) + Q(21) + Q(22);
                double rapnoy = fmax((Q(4) - Q(14) - Q(18) - Q(20)), 0.) / totmas;
                H(7) = H(7) * rapnoy;
                H(8) = H(8) * rapnoy;
                H(10) = H(10) * rapnoy;
                H(13) = H(13) * rapnoy;
                Q(5) = Q(5) * rapnoy;
                Q(6) = Q(6) * rapnoy;
                Q(21) = Q(21) * rapnoy;
                Q(22) = Q(22) * rapnoy;
                totmas = Q(19) + Q(20) + Q(24) + Q(26) + Q(27);
                double rapbry = Q(41) / totmas;
                H(9) = H(9) * rapbry;
                H(12) = H(12) * rapbry;
                Q(19) = Q(19) * rapbry;
                Q(20) = Q(20) * rapbry;
                Q(24) = Q(24) * rapbry;
                Q(26) = Q(26) * rapbry;
                Q(27) = Q(27) * rapbry;
#undef Q
#undef H
            }
}

/* ============================================================================
 * clamps, F:431-450
 * ========================================================================== */
void orc_clamp(const orc_grid* g, int ilat0, int ilat1, double* qj1) {
    for (int m = 0; m < NBCON - 1; m++)
        for (int k = 0; k < g->niv; k++)
            for (int j = ilat0; j <= ilat1; j++)
                for (int i = 0; i < g->nlon; i++) G4(qj1, i, j, k, m) = fmax(G4(qj1, i, j, k, m), 1.e-30);
    for (int k = g->nivbas; k < g->niv; k++)
        for (int j = ilat0; j <= ilat1; j++)
            for (int i = 0; i < g->nlon; i++) G4(qj1, i, j, k, NBCON - 1) = G4(qj1, i, j, k, 4);
}

/* ============================================================================
 * the chemistry block of the time loop, F:398-450
 * ========================================================================== */
int orc_step(const orc_grid* g, int ilat0, int ilat1, double daynum, double dt, const double* alt,
             const double* trajlon, const double* trajlat, const double* trajpre, const double* trajtem, int irapp,
             double* qj1, double* hc, double* vsed3d, double* parth2osed, double* parthno3sed, double* surfarea,
             double* sza3d, int fuse, double* diag, int nthreads) {
    int pmax = 0;
    const int nblk_lon = (g->nlon + ORC_BLOCK - 1) / ORC_BLOCK;
    const int ntask = (ilat1 - ilat0 + 1) * nblk_lon;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt) reduction(max : pmax)
#endif
    {
        work* wfull = work_alloc(ORC_BLOCK, g->nivbas);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int task = 0; task < ntask; task++) {
            int j = ilat0 + task / nblk_lon;
            int i0 = (task % nblk_lon) * ORC_BLOCK;
            int nl = g->nlon - i0 < ORC_BLOCK ? g->nlon - i0 : ORC_BLOCK;
            work* w = wfull;
            if (nl != ORC_BLOCK) w = work_alloc(nl, g->nivbas);
            int p = orc_chem3d_block(g, w, j, i0, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1,
                                     hc, vsed3d, parth2osed, parthno3sed, surfarea, sza3d, diag);
            if (p > pmax) pmax = p;
            if (w != wfull) work_free(w);
        }
        work_free(wfull);
    }
    (void)nthreads;
    if (fuse) {
        orc_conserv(g, ilat0, ilat1, qj1, hc);
        orc_clamp(g, ilat0, ilat1, qj1);
    }
    return pmax;
}
