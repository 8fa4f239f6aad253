/*
 * column_oracle.cpp — CPU FP64 oracle of the column physics around the
 * chemistry step: sedimentation, tropospheric forcing, altitude.
 *
 * TEST INFRASTRUCTURE ONLY: the tests call it as the checker of the CUDA
 * kernels in reprobus_gb300/csrc/column_kernels.cu; the product library never
 * links or calls it.
 *
 * PARITY UNPINNED (as for chem_oracle.c): the reference is Fortran with no
 * compiler here and ships no tests or fixtures. Each function restates the
 * reference routine loop by loop, in the reference's loop order and
 * evaluation order (F = src/reprobus_l137_20230723.f), compiled without FMA
 * contraction.
 *
 * Arrays: FP64, Fortran layout (lon fastest); A3(a,i,j,k) indexes a
 * (nlon,nlat,*) array with 1-based i, j, k. C++ only for the shared table of
 * the reference's forcing data (tropo_tables.h); the functions are C-ABI.
 */
#include <math.h>
#include <stddef.h>
#include <string.h>

#include "../reprobus_gb300/csrc/tropo_tables.h"

extern "C" {

#define A3(a, i, j, k) (a)[((size_t)(i) - 1) + (size_t)nlon * (((size_t)(j) - 1) + (size_t)nlat * ((size_t)(k) - 1))]
#define A2(a, i, j) (a)[((size_t)(i) - 1) + (size_t)nlon * ((size_t)(j) - 1)]

/* sedimentation, F:2416-2522, latitude rows ilat0..ilat1 (1-based).
 * pre/tem: the irapp slices of trajpre/trajtem (nlon,nlat,niv); qj1
 * (nlon,nlat,niv,43); vsed/ph2o/pno3 (nlon,nlat,nivbas). hnm is kept per
 * level as the reference's hnm(nlon,nivbas) array is. */
void orc_sedimentation(int nlon, int nlat, int niv, int nivbas, int nivhau, int ilat0, int ilat1,
                       const double* pre, const double* tem, double* qj1, const double* vsed, int nivh2o,
                       const double* ph2o, const double* pno3, double dt) {
    const size_t p3 = (size_t)nlon * nlat * niv;
    double* q3 = qj1 + 2 * p3;
    double* q4 = qj1 + 3 * p3;
    double* q5 = qj1 + 4 * p3;
    for (int ilat = ilat0; ilat <= ilat1; ilat++) {
        /* F:2443-2448 */
#define HNM(i, k) (A3(pre, i, ilat, k) / (A3(tem, i, ilat, k) * 1.38e-19))
        /* F:2456-2480 */
        for (int iniv = nivh2o - 1; iniv >= nivhau; iniv--) {
            for (int ilon = 1; ilon <= nlon; ilon++) {
                const double dz = 7000. * log(A3(pre, ilon, ilat, iniv) / A3(pre, ilon, ilat, iniv - 1));
                double fracup = A3(vsed, ilon, ilat, iniv - 1) * dt / dz;
                double fracdown = A3(vsed, ilon, ilat, iniv) * dt / dz;
                fracup = fmin(fracup, 1.0);
                fracdown = fmin(fracdown, 1.0);
                A3(q3, ilon, ilat, iniv) = A3(q3, ilon, ilat, iniv) +
                                           A3(q3, ilon, ilat, iniv - 1) * (1. - A3(ph2o, ilon, ilat, iniv - 1)) *
                                               HNM(ilon, iniv - 1) / HNM(ilon, iniv) * fracup -
                                           A3(q3, ilon, ilat, iniv) * (1. - A3(ph2o, ilon, ilat, iniv)) * fracdown;
            }
        }
        /* F:2482-2514 */
        for (int iniv = nivbas; iniv >= nivhau; iniv--) {
            for (int ilon = 1; ilon <= nlon; ilon++) {
                const double dz = 7000. * log(A3(pre, ilon, ilat, iniv) / A3(pre, ilon, ilat, iniv - 1));
                double fracup = A3(vsed, ilon, ilat, iniv - 1) * dt / dz;
                double fracdown = A3(vsed, ilon, ilat, iniv) * dt / dz;
                fracup = fmin(fracup, 1.0);
                fracdown = fmin(fracdown, 1.0);
                A3(q4, ilon, ilat, iniv) = A3(q4, ilon, ilat, iniv) +
                                           A3(q5, ilon, ilat, iniv - 1) * (1. - A3(pno3, ilon, ilat, iniv - 1)) *
                                               HNM(ilon, iniv - 1) / HNM(ilon, iniv) * fracup -
                                           A3(q5, ilon, ilat, iniv) * (1. - A3(pno3, ilon, ilat, iniv)) * fracdown;
                A3(q5, ilon, ilat, iniv) = A3(q5, ilon, ilat, iniv) +
                                           A3(q5, ilon, ilat, iniv - 1) * (1. - A3(pno3, ilon, ilat, iniv - 1)) *
                                               HNM(ilon, iniv - 1) / HNM(ilon, iniv) * fracup -
                                           A3(q5, ilon, ilat, iniv) * (1. - A3(pno3, ilon, ilat, iniv)) * fracdown;
            }
        }
#undef HNM
    }
}

/* the date interpolation of tropo, F:4414-4495; returns 0, or -1 for dates
 * outside the tables. v: the 16 values in the order of the slots
 * 1 2 4 7 31..42 (F:4502-4518). */
int orc_tropo_values(int ian, int imois, double* v) {
    const double yearccmval = (double)ian + (double)(imois - 1) / 12.;
    double s[rpb::TROPO_NTAB];
    int icount = 0, found = 0;
    for (int iyear = 1988; iyear <= 2024; iyear++) {
        icount = icount + 1;
        if ((double)iyear + 0.5 > yearccmval) {
            if (icount == 1) return -1;
            const double cinf = (yearccmval - (double)(iyear - 1) - 0.5) / 1.;
            const double csup = 1. - cinf;
            for (int n = 0; n < rpb::TROPO_NTAB; n++)
                s[n] = cinf * rpb::kTropoTab[n][icount - 1] + csup * rpb::kTropoTab[n][icount - 2];
            found = 1;
            break;
        }
    }
    if (!found) return -1;
    s[rpb::TT_CFC12] = s[rpb::TT_CFC12] + s[rpb::TT_CFC114] + 0.5 * s[rpb::TT_CFC115];
    s[rpb::TT_CH3CCL3] = s[rpb::TT_CH3CCL3] + s[rpb::TT_HCFC141B] * 2. / 3.;
    s[rpb::TT_HCFC22] = s[rpb::TT_HCFC22] + s[rpb::TT_HCFC142B];
    s[rpb::TT_H1301] = s[rpb::TT_H1301] + s[rpb::TT_H2402] * 2.;
    const int order[16] = {rpb::TT_N2O,    rpb::TT_CH4,   rpb::TT_NOY,    rpb::TT_CLY,   rpb::TT_CFC11, rpb::TT_CFC12,
                           rpb::TT_CFC113, rpb::TT_CCL4,  rpb::TT_CH3CCL3, rpb::TT_CH3CL, rpb::TT_HCFC22, rpb::TT_CH3BR,
                           rpb::TT_H1211,  rpb::TT_H1301, rpb::TT_BRY,    rpb::TT_CH2BR2};
    for (int n = 0; n < 16; n++) v[n] = s[order[n]];
    return 0;
}

/* tropo, co_tropo and ecmwfh2o for rows ilat0..ilat1 (F:4498-4571,
 * F:4617-4636, F:8649-8655), in the reference's order. v: orc_tropo_values;
 * co (nlon,nlat) or NULL; hj1 (nlon,nlat,niv) or NULL. */
void orc_forcing(int nlon, int nlat, int niv, int nivbas, int ilat0, int ilat1, const double* v, double dt,
                 const double* pre, const double* co, const double* hj1, int nivh2o, double* qj1, double* hc) {
    const size_t p3 = (size_t)nlon * nlat * niv;
    static const int slot[16] = {1, 2, 4, 7, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42};
    /* tropo: F:4498-4519 */
    for (int iniv = nivbas + 1; iniv <= niv; iniv++)
        for (int ilat = ilat0; ilat <= ilat1; ilat++)
            for (int ilon = 1; ilon <= nlon; ilon++)
                for (int n = 0; n < 16; n++) A3(qj1 + p3 * (slot[n] - 1), ilon, ilat, iniv) = v[n];
    /* F:4527-4543 */
    {
        const double tau = 1.;
        const double dtt = dt / (24. * 60. * 60.);
        double* q8 = qj1 + 7 * p3;
        for (int iniv = nivbas + 1; iniv <= niv; iniv++)
            for (int ilat = ilat0; ilat <= ilat1; ilat++)
                for (int ilon = 1; ilon <= nlon; ilon++) {
                    double ilim;
                    if (A3(pre, ilon, ilat, iniv) > 370.)
                        ilim = -2.3825e-8 * log(A3(pre, ilon, ilat, iniv)) + 1.9457e-7;
                    else
                        ilim = A3(q8, ilon, ilat, iniv);
                    A3(q8, ilon, ilat, iniv) = fmax(ilim + (A3(q8, ilon, ilat, iniv) - ilim) * exp(-dtt / tau), 0.);
                }
    }
    /* F:4548-4555 */
    for (int iniv = nivbas; iniv <= niv; iniv++)
        for (int ilat = ilat0; ilat <= ilat1; ilat++)
            for (int ilon = 1; ilon <= nlon; ilon++) {
                A3(hc + 4 * p3, ilon, ilat, iniv) = A3(qj1 + 7 * p3, ilon, ilat, iniv);
                A3(qj1 + 10 * p3, ilon, ilat, iniv) = A3(qj1 + 7 * p3, ilon, ilat, iniv);
            }
    /* co_tropo: F:4612-4636 */
    if (co) {
        const double tau = 24.;
        const double dtt = dt / (60. * 60.);
        double* q9 = qj1 + 8 * p3;
        for (int iniv = nivbas + 1; iniv <= niv; iniv++)
            for (int ilat = ilat0; ilat <= ilat1; ilat++)
                for (int ilon = 1; ilon <= nlon; ilon++) {
                    const double ilim = A2(co, ilon, ilat);
                    A3(q9, ilon, ilat, iniv) = fmax(ilim + (A3(q9, ilon, ilat, iniv) - ilim) * exp(-dtt / tau), 1.e-30);
                }
    }
    /* ecmwfh2o: F:8649-8655 */
    if (hj1)
        for (int iniv = nivh2o; iniv <= niv; iniv++)
            for (int ilat = ilat0; ilat <= ilat1; ilat++)
                for (int ilon = 1; ilon <= nlon; ilon++)
                    A3(qj1 + 2 * p3, ilon, ilat, iniv) = A3(hj1, ilon, ilat, iniv) * 28.97 / 18.;
}

/* altitude, altitude.f90:1-148, with the nearest regular point taken on a
 * grid of spacing 360/nlon x 180/(nlat-1) (the reference writes 2. for its
 * 2 x 2 degree grid) and its latitude index kept inside 1..nlat.
 * t, h2o: regular grid (nlon,nlat,niv); trajlon/lat/pre: one slice. */
void orc_altitude(int nlon, int nlat, int niv, const double* relief, const double* psol, const double* aaa,
                  const double* bbb, const double* t, const double* h2o, const double* trajlon,
                  const double* trajlat, const double* trajpre, double* alt, double* work /* 3 nlon nlat niv */,
                  int* iwork /* 3 nlon nlat niv */) {
    const size_t n3 = (size_t)nlon * nlat * niv;
    double* p = work;
    double* georeg = work + n3;
    double* tv = work + 2 * n3;
    int* indlon = iwork;
    int* indlat = iwork + n3;
    int* indpre = iwork + 2 * n3;
    double* geo = alt; /* geo lives in alt until the last loop */
    const double ctegas = 287.04 / 9.80665;
    const double pi = 2. * asin(1.);
    const double dlon = 360. / nlon, dlat = 180. / (nlat - 1);
    /* :34-40 */
    for (int iniv = 1; iniv <= niv; iniv++)
        for (int ilat = 1; ilat <= nlat; ilat++)
            for (int ilon = 1; ilon <= nlon; ilon++)
                A3(p, ilon, ilat, iniv) = aaa[iniv - 1] + bbb[iniv - 1] * A2(psol, ilon, ilat);
    /* :45 */
    for (size_t i = 0; i < n3; i++) tv[i] = t[i] * (1. + 0.608 * h2o[i] * 18. / 28.97);
    /* :51-57 */
    for (int ilat = 1; ilat <= nlat; ilat++)
        for (int ilon = 1; ilon <= nlon; ilon++)
            A3(georeg, ilon, ilat, niv) = A2(relief, ilon, ilat) + ctegas * A3(tv, ilon, ilat, niv) *
                                                                      log(A2(psol, ilon, ilat) / A3(p, ilon, ilat, niv)) * 1.e-3;
    for (int iniv = niv - 1; iniv >= 1; iniv--)
        for (int ilat = 1; ilat <= nlat; ilat++)
            for (int ilon = 1; ilon <= nlon; ilon++)
                A3(georeg, ilon, ilat, iniv) =
                    A3(georeg, ilon, ilat, iniv + 1) +
                    ctegas * ((A3(tv, ilon, ilat, iniv + 1) + A3(tv, ilon, ilat, iniv)) / 2.) *
                        log(A3(p, ilon, ilat, iniv + 1) / A3(p, ilon, ilat, iniv)) * 1.e-3;
    /* :61-74 (nint: round half away from zero) */
    for (size_t i = 0; i < n3; i++) {
        indlon[i] = (int)round(trajlon[i] / dlon) + 1;
        if (indlon[i] > nlon) indlon[i] = 1;
        if (indlon[i] < 1) indlon[i] = 1;
        indlat[i] = (int)round((90. - trajlat[i]) / dlat) + 1;
        if (indlat[i] < 1) indlat[i] = 1;
        if (indlat[i] > nlat) indlat[i] = nlat;
    }
    /* :76-87 — pirr kept in tv's place would alias; use a local per point */
    /* :90-106 */
    for (size_t i = 0; i < n3; i++) {
        const int ilr = indlon[i], jlr = indlat[i];
        double pirr = fmax(trajpre[i], A3(p, ilr, jlr, 1));
        pirr = fmin(trajpre[i], A3(p, ilr, jlr, niv));
        for (int inivreg = niv; inivreg >= 2; inivreg--)
            if (A3(p, ilr, jlr, inivreg) >= pirr) {
                geo[i] = A3(georeg, ilr, jlr, inivreg);
                indpre[i] = inivreg;
            }
        /* :108-122 */
        const int kr = indpre[i];
        const double dz = ctegas * (A3(tv, ilr, jlr, kr) + A3(tv, ilr, jlr, kr - 1)) / 2. *
                          log(A3(p, ilr, jlr, kr) / pirr) * 1.e-3;
        geo[i] = geo[i] + dz;
    }
    /* :126-146 */
    for (size_t i = 0; i < n3; i++) {
        const double xlat = trajlat[i] * pi / 180.;
        alt[i] = (1. + 0.002644 * cos(2. * xlat)) * geo[i] + (1. + 0.0089 * cos(2. * xlat)) * (geo[i] * geo[i]) / 6245.;
    }
}

}  /* extern "C" */
