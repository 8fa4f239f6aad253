// chem_cell.cuh — per-cell FP64 device code of the REPROBUS chemistry step.
//
// One CUDA thread owns one grid cell. Every function restates a block of the
// reference (src/reprobus_l137_20230723.f "F:", src/jno.f90 "JNO:") for a
// single cell, keeping the Fortran evaluation order of each expression; the
// only reordering is between cells (the reference loops over longitude inside
// each block, here each thread runs the blocks in sequence for its cell,
// which is the same arithmetic because every block is elementwise in
// (lon, level)). The vertical prefix sums of total (F:5153-5186) and jno
// (JNO:107-126) are computed per column by k_columns before the cell kernel.
// On GB300 every FP64 operation is scarce (2 per clock per SM), so the rate
// stage divides by a constant as a product with its reciprocal (within an
// ulp of the quotient), takes its exponentials from exp64 (exp64.cuh, within
// 1.5 ulp), its logarithms from log64 (log64.cuh, within 1.6 ulp) and the
// quotients of the rate constants and of the liquid aerosol from div64
// (div64.cuh, within an ulp).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "chem_enums.h"
#include "div64.cuh"
#include "exp64.cuh"
#include "log64.cuh"

namespace rpb {

constexpr int NBCON = 43;
constexpr int NCM = 15;
constexpr int NPHOT = 41;
constexpr int NZ = 101;
constexpr int NSZA = 27;
constexpr int NOZO = 7;
constexpr int NRATE = 99;
constexpr double PI = 3.141592653589793;  // 2.*asin(1.0), F:2750
constexpr double LN10 = 2.302585092994046;  // 10^y evaluated as exp(y ln 10)
// transcendental constants of the aerosol and rate code, evaluated once here:
// ln 760 (F:2866), ln 0.6 (Troe broadening, F:920), and for the log-normal
// liquid aerosol of width sigma = 1.8 (F:2632, F:3091-3096)
// exp(-4.5 ln^2 sigma), exp(0.5 ln^2 sigma), exp(2 ln^2 sigma)
constexpr double LN760 = 6.633318433280377, LN06 = -0.5108256237659907;
constexpr double AER_EXP_M45 = 0.21124868545437422, AER_EXP_05 = 1.18856486285036,
                 AER_EXP_2 = 1.9956829585543872;

// per-step constants shared by all cells
struct StepConst {
    double ut, eqh, srd, crd;  // zenith: UT hour, equation of time (h), sin/cos(declination)
    double dt;
    double troe[18];           // COMMON /constant/
    double ltroe[18];          // ln troe[i] (0 where troe[i] <= 0)
};

// ----------------------------------------------------------------------------
// zenith, F:5382-5403 (per cell; the per-step part F:5340-5380 is in StepConst)
// ----------------------------------------------------------------------------
__device__ __forceinline__ double cell_zenith(const StepConst& sc, double lon, double lat) {
    double rlt = lat * PI * (1. / 180.);
    double lbut = 12. - sc.eqh - lon * 24. * (1. / 360.);
    double lzut = 15. * (sc.ut - lbut);
    double zpt = lzut * PI * (1. / 180.);
    double srlt, crlt;
    sincos(rlt, &srlt, &crlt);
    double csz = srlt * sc.srd + crlt * sc.crd * cos(zpt);
    double zr = acos(csz);
    double s = zr * (180. / PI);
    return fmax(s, 0.);
}

// ----------------------------------------------------------------------------
// phot, F:5060-5134 — 40 J values by trilinear interpolation (sunlit cells)
// ajl is the Fortran-order table ajl(40,101,27,7); alt in km.
// ----------------------------------------------------------------------------
__constant__ double c_dsza[NSZA] = {0.,  5.,  10., 15., 20., 25., 30., 35., 40., 45., 50., 55., 60., 65.,
                                    70., 75., 80., 82., 84., 86., 88., 90., 91., 92., 93., 94., 95.};
__constant__ double c_xv3[NOZO] = {0.4, 0.6, 0.8, 1.0, 1.2, 1.4, 1.6};

__device__ __forceinline__ void cell_phot(const double* __restrict__ ajl, const double* __restrict__ o3up,
                                          double alt, double sza, double o3t, double* tj) {
    // is: first SZA node >= sza, minus one, capped at nsza-1 (F:5055-5068)
    int is = NSZA - 1;
#pragma unroll 1
    for (int i = 1; i <= NSZA; i++) {
        if (c_dsza[i - 1] >= sza) { is = i - 1; break; }
    }
    const double dz = 1.;
    const double stepo3 = div64(c_xv3[NOZO - 1] - c_xv3[0], (double)(NOZO - 1));
    double zin = fmin(alt, 78.9);
    int iz = (int)(zin / dz) + 1;
    int ii = (int)zin;
    double v3std = o3up[ii] - (zin - (double)ii) * (o3up[ii] - o3up[ii + 1]);
    double v3rat = div64(o3t, v3std);
    v3rat = fmax(v3rat, c_xv3[0]);
    v3rat = fmin(v3rat, c_xv3[NOZO - 1]);
    int iv = (int)trunc(div64(v3rat - c_xv3[0], stepo3)) + 1;
    iv = min(iv, NOZO - 1);
    int j = max(iz, 1);
    int k = max(is, 1);
    int l = max(iv, 1);
    double cizin = (zin - (double)(j - 1) * dz) / dz;
    double cisza = div64(sza - c_dsza[k - 1], c_dsza[k] - c_dsza[k - 1]);
    double cio3t = div64(v3rat - c_xv3[l - 1], c_xv3[l] - c_xv3[l - 1]);
    double w111 = (1. - cizin) * (1. - cisza) * (1. - cio3t);
    double w112 = (1. - cizin) * (1. - cisza) * cio3t;
    double w121 = (1. - cizin) * cisza * (1. - cio3t);
    double w122 = (1. - cizin) * cisza * cio3t;
    double w211 = cizin * (1. - cisza) * (1. - cio3t);
    double w212 = cizin * (1. - cisza) * cio3t;
    double w221 = cizin * cisza * (1. - cio3t);
    double w222 = cizin * cisza * cio3t;
    // corner (j,k,l) 1-based -> base offset of ajl(1, j, k, l)
    const size_t sj = (NPHOT - 1), sk = (size_t)(NPHOT - 1) * NZ, sl = (size_t)(NPHOT - 1) * NZ * NSZA;
    const double2* p111 = (const double2*)(ajl + (j - 1) * sj + (k - 1) * sk + (l - 1) * sl);
    const double2* p112 = (const double2*)((const double*)p111 + sl);
    const double2* p121 = (const double2*)((const double*)p111 + sk);
    const double2* p122 = (const double2*)((const double*)p111 + sk + sl);
    const double2* p211 = (const double2*)((const double*)p111 + sj);
    const double2* p212 = (const double2*)((const double*)p111 + sj + sl);
    const double2* p221 = (const double2*)((const double*)p111 + sj + sk);
    const double2* p222 = (const double2*)((const double*)p111 + sj + sk + sl);
#pragma unroll 4
    for (int q = 0; q < (NPHOT - 1) / 2; q++) {
        double2 a = __ldg(p111 + q), b = __ldg(p112 + q), c = __ldg(p121 + q), d = __ldg(p122 + q);
        double2 e = __ldg(p211 + q), f = __ldg(p212 + q), g = __ldg(p221 + q), h = __ldg(p222 + q);
        tj[2 * q] = w111 * a.x + w112 * b.x + w121 * c.x + w122 * d.x + w211 * e.x + w212 * f.x + w221 * g.x +
                    w222 * h.x;
        tj[2 * q + 1] = w111 * a.y + w112 * b.y + w121 * c.y + w122 * d.y + w211 * e.y + w212 * f.y +
                        w221 * g.y + w222 * h.y;
    }
}

// ----------------------------------------------------------------------------
// jno, JNO:132-245 for one cell; colo2/colno/colo3 are the column sums of
// JNO:109-126 at this level, sza_top the zenith angle of level 1 (JNO:139).
// ----------------------------------------------------------------------------
__constant__ double c_jno_so2[3][6] = {{1.12e-23, 2.45e-23, 7.19e-23, 3.04e-22, 1.75e-21, 1.11e-20},
                                       {1.35e-22, 2.99e-22, 7.33e-22, 3.07e-21, 1.69e-20, 1.66e-19},
                                       {2.97e-22, 5.83e-22, 2.05e-21, 8.19e-21, 4.80e-20, 2.66e-19}};
__constant__ double c_jno_sno1[3][6] = {{0.00e+00, 1.32e-18, 6.35e-19, 7.09e-19, 2.18e-19, 4.67e-19},
                                        {0.00e+00, 0.00e+00, 3.05e-21, 5.76e-19, 2.29e-18, 2.21e-18},
                                        {1.80e-18, 1.50e-18, 5.01e-19, 7.20e-20, 6.72e-20, 1.49e-21}};
__constant__ double c_jno_sno2[3][6] = {{0.00e+00, 4.41e-17, 4.45e-17, 4.50e-17, 2.94e-17, 4.35e-17},
                                        {0.00e+00, 0.00e+00, 3.20e-21, 5.71e-17, 9.09e-17, 6.00e-17},
                                        {1.40e-16, 1.52e-16, 7.00e-17, 2.83e-17, 2.73e-17, 6.57e-18}};
__constant__ double c_jno_w1[3][6] = {{0.00e+00, 5.12e-02, 1.36e-01, 1.65e-01, 1.41e-01, 4.50e-02},
                                      {0.00e+00, 0.00e+00, 1.93e-03, 9.73e-02, 9.75e-02, 3.48e-02},
                                      {4.50e-02, 1.80e-01, 2.25e-01, 2.25e-01, 1.80e-01, 4.50e-02}};
__constant__ double c_jno_w2[3][6] = {{0.00e+00, 5.68e-03, 1.52e-02, 1.83e-02, 1.57e-02, 5.00e-03},
                                      {0.00e+00, 0.00e+00, 2.14e-04, 1.08e-02, 1.08e-02, 3.86e-03},
                                      {5.00e-03, 2.00e-02, 2.50e-02, 2.50e-02, 2.00e-02, 5.00e-03}};
__constant__ double c_jno_dl[3] = {2.3, 1.5, 1.5};
__constant__ double c_jno_i0[3] = {3.98e+11, 2.21e+11, 2.30e+11};
__constant__ double c_jno_so3[3] = {4.6e-19, 6.7e-19, 7.1e-19};

__device__ __forceinline__ double cell_jno(double sza_top, double hnm, double colo2, double colno, double colo3) {
    const double factor = 3.141592 / 180.;
    const double d = 1.65e+09, a = 5.1e+07, kq = 1.5e-09;
    double sec = div64(1., cos(sza_top * factor));
    colo2 = colo2 * sec;
    colno = colno * sec;
    colo3 = colo3 * sec;
    double n2 = hnm * 0.78;
    double p = div64(d, a + d + kq * n2);
    double bd[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        double to3 = exp64(-c_jno_so3[b] * colo3);
        double sum = 0.;
#pragma unroll
        for (int s = 0; s < 6; s++) {
            double term = exp64(-c_jno_so2[b][s] * colo2) *
                          (c_jno_w1[b][s] * c_jno_sno1[b][s] * exp64(-c_jno_sno1[b][s] * colno) +
                           c_jno_w2[b][s] * c_jno_sno2[b][s] * exp64(-c_jno_sno2[b][s] * colno));
            sum = (s == 0) ? term : sum + term;
        }
        bd[b] = c_jno_dl[b] * c_jno_i0[b] * to3 * p * sum;
    }
    return fmax(bd[0] + bd[1] + bd[2], 1.e-30);
}

// ----------------------------------------------------------------------------
// analytic (F:2620-3361) + density (F:4033-4073) + hetero (F:3365-4029) for
// one cell of levels nivhau..nivbas. ck: number densities at step start.
// ----------------------------------------------------------------------------
struct Aerosol {
    double het[9];
    double parthno3, parthno3sl, parth2o, parthcl;
    double vsed, surf;
};

__constant__ double c_an_a1[3] = {12.37208932, 11.820654354, -180.06541028};
__constant__ double c_an_b1[3] = {-0.16125516114, -0.20786404244, -0.38601102592};
__constant__ double c_an_c1[3] = {-30.490657554, -4.807306373, -93.317846778};
__constant__ double c_an_d1[3] = {-2.1133114241, -5.1727540348, 273.88132245};
__constant__ double c_an_a2[3] = {13.455394705, 12.891938068, -176.95814097};
__constant__ double c_an_b2[3] = {-0.1921312255, -0.232338847708, -0.36257048154};
__constant__ double c_an_c2[3] = {-34.285174607, -6.4261237757, -90.469744201};
__constant__ double c_an_d2[3] = {-1.7620073078, -4.9005471319, 267.45509988};
__constant__ double c_an_bnre[7] = {-3.18657, 0.992696, -0.153193e-2, -0.987059e-3, -0.578878e-3, 0.855176e-4,
                                    -0.327815e-5};
// Carslaw et al. (1995) coefficients, 1-based in the formulas below
__constant__ double c_an_qn[11] = {0., 14.5734, 0.0615994, -1.14895, 0.691693, -0.098863,
                                   0.0051579, 0.123472, -0.115574, 0.0110113, 0.0097914};
__constant__ double c_an_qs[11] = {0., 14.4700, 0.0638795, -3.29597, 1.778224, -0.223244,
                                   0.0086486, 0.536695, -0.335164, 0.0265153, 0.0157550};
__constant__ double c_an_kn[8] = {0., -39.136, 6358.4, 83.29, -17650.0, 198.53, -11948, -28.469};
__constant__ double c_an_ks[8] = {0., -21.661, 2724.2, 51.81, -15732.0, 47.004, -6969.0, -4.6183};
__constant__ double c_dens_x[23] = {0., 2.393284E-02, -4.359335E-05, 7.961181E-08, 0.0, -0.198716351,
                                    1.39564574E-03, -2.020633E-06, 0.51684706, -3.0539E-03, 4.505475E-06,
                                    -0.30119511, 1.840408E-03, -2.7221253742E-06, -0.11331674116, 8.47763E-04,
                                    -1.22336185E-06, 0.3455282, -2.2111E-03, 3.503768245E-06, -0.2315332,
                                    1.60074E-03, -2.5827835E-06};

static __device__ __noinline__ void cell_aerosol(double temp, double ptot, double hnm, const double* ck, Aerosol& A) {
    const double r = 8.205e-5;
    const double* qn = c_an_qn;
    const double* qs = c_an_qs;
    const double* kn = c_an_kn;
    const double* ks = c_an_ks;
    const double ndrop = 10.;
    const double nnat_small_max = 1.;
    const double rnats = 0.5e-4, rnatl = 6.5e-4, rice = 10.e-4;
    const double amu = 1.66e-24;
    // initialisation F:2753-2776
    double rmean = 0., aliq = 0., nnats = 0., nnatl = 0., anat = 0., nice = 0., aice = 0.;
    int lnat = 0, lice = 0, condliq = 0;
    double vnat = 0., vnatl = 0.;
    double parthno3l = 1., parthno3s = 1.;
    A.vsed = 0.;
    A.parthno3 = 1.;
    A.parthno3sl = 1.;
    A.parth2o = 1.;
    A.parthcl = 1.;
    // F:2778-2787
    const double rhnm = div64(1., hnm);
    double qh2o = ck[2] * rhnm;
    double pw = qh2o * ptot * (1. / 1013.0);
    pw = fmin(pw, 2.e-3 / 1013.);
    double qhno3 = ck[4] * rhnm;
    double pn0 = qhno3 * ptot * (1. / 1013.0);
    // NAT F:2795-2857
    {
        double t = fmin(temp, 273.);
        double pn0t = pn0 * 1013. * 0.75;
        double zmt = -2.7836 - 0.00088 * t;
        double zbt = 38.9855 - div64(11397.0, t) + 0.009179 * t;
        double zhno3eq = exp64(zmt * log64(pw * 1013. * 0.75) + zbt * LN10);
        if (div64(pn0t, zhno3eq) >= 1.) {
            lnat = 1;
            double pn = zhno3eq * (1. / (0.75 * 1013.));
            double hno3s = div64((pn0 - pn) * 1013. * hnm, ptot);
            hno3s = fmax(hno3s, 0.);
            vnat = hno3s * amu * 117. * (1. / 1.35);
            double vnat_small_max = nnat_small_max * (4. / 3. * PI * (rnats * rnats * rnats));
            if (vnat > vnat_small_max) {
                nnats = nnat_small_max;
                nnatl = (vnat - vnat_small_max) * (1. / (4. / 3. * PI * (rnatl * rnatl * rnatl)));
                vnatl = vnat - vnat_small_max;
            } else {
                nnats = vnat * (1. / (4. / 3. * PI * (rnats * rnats * rnats)));
                nnatl = 0.;
                vnatl = 0.;
            }
            anat = nnats * 4 * PI * (rnats * rnats) + nnatl * 4 * PI * (rnatl * rnatl);
            parthno3s = 1.0 - div64(pn0 - pn, pn0);
            parthno3s = fmax(parthno3s, 0.);
            parthno3s = fmin(parthno3s, 1.);
            A.parthno3sl = 1.0 - div64(div64((pn0 - pn) * vnatl, vnat), pn0);
            A.parthno3sl = fmax(A.parthno3sl, 0.);
            A.parthno3sl = fmin(A.parthno3sl, 1.);
        }
    }
    // ice F:2861-2913
    double tice;
    {
        double t = fmin(temp, 273.);
        tice = div64(2668.70, 10.4310 - (log64(pw) + LN760) * (1. / LN10));
        if (t <= tice) {
            lice = 1;
            lnat = 0;
            anat = 0.;
            double zh2oeq = exp64((div64(-2668.7, t) + 10.4310) * LN10);
            double ph2o = zh2oeq * (1. / 760.0);
            double h2os = div64(fmax(pw - ph2o, 0.) * 1013. * hnm, ptot);
            double vice = h2os * amu * 18. * (1. / 0.928);
            nice = vice * (1. / (4. / 3. * PI * (rice * rice * rice)));
            aice = nice * 4 * PI * (rice * rice);
            A.parth2o = 1.0 - div64(fmax(pw - ph2o, 0.), pw);
            A.parth2o = fmax(A.parth2o, 0.);
            A.parth2o = fmin(A.parth2o, 1.);
            double zmt = -2.7836 - 0.00088 * t;
            double zbt = 38.9855 - div64(11397.0, t) + 0.009179 * t;
            double zhno3eq = exp64(zmt * log64(pw * A.parth2o * 1013. * 0.75) + zbt * LN10);
            double pn = zhno3eq * (1. / (0.75 * 1013.));
            parthno3s = 1.0 - div64(pn0 - pn, pn0);
            parthno3s = fmax(parthno3s, 0.);
            parthno3s = fmin(parthno3s, 1.);
            A.parthno3sl = parthno3s;
        }
    }
    // liquid aerosols F:2919-3056
    double ns, ms, ws, wn;
    double tl = fmax(temp, fmax(tice - 3.0, 185.));
    {
        condliq = 1;
        double t = tl;
        const double rt = div64(1., t);  // E / T as E * (1 / T) in the liquid-aerosol blocks
        double qh2ol = ck[2] * A.parth2o * rhnm;
        pw = qh2ol * ptot * (1. / 1013.0);
        pw = fmin(pw, 2.e-3 / 1013.);
        pw = fmax(pw, 2.e-5 / 1013.);
        double qh2so4 = fmax(ck[11] * rhnm, 1.e-18);
        ns = ptot * 100.0 * qh2so4 * (1. / 8.314) * rt;
        double qhno3l = ck[4] * parthno3s * rhnm;
        pn0 = ptot * (1. / 1013.0) * qhno3l;
        double a = ks[3] + ks[4] * rt;
        double b = ks[1] + ks[2] * rt;
        double cq = ks[5] + ks[6] * rt + ks[7] * log64(t) - log64(pw);
        double det = b * b - 4. * a * cq;
        double msb;
        if (det > 0.) {
            double xsb = div64(-b - sqrt64(det), 2. * a);
            msb = div64(55.51 * xsb, 1.0 - xsb);
        } else {
            msb = 0.;
            condliq = 0;
        }
        ms = msb;
        ws = div64(msb * 0.098076, 1.0 + msb * 0.098076);
        wn = 0.0;
        double wts = fmax(41., ws * 100.);
        double wd = wts - 40.;
        double muh2so4 = 4.184 * (1.514e4 - 286. * wd + 1.08 * (wd * wd) - div64(3941., exp64(0.1 * log64(wd))));
        double ph2so4 = exp64(-10156. * rt + 16.2590 - muh2so4 * (rt * (1. / 8.314)));
        if (qh2so4 * ptot * (1. / 1013.) <= ph2so4) {
            ms = 0.;
            ws = 0.;
            condliq = 0;
        }
        if (condliq == 1 && t < 215.) {
            double tf = t;
            double tt = r * tf * ns;
            double tr = 1.0e4 * rt - 43.4782608;
            double pr = log64(pw) + 18.4;
            double tr2 = tr * tr, tr3 = tr2 * tr, pr2 = pr * pr, pr3 = pr2 * pr;
            double hsb = qs[1] + qs[2] * tr2 + (qs[3] + qs[4] * tr + qs[5] * tr2 + qs[6] * tr3) * pr +
                         (qs[7] + qs[8] * tr + qs[9] * tr2) * pr2 + qs[10] * tr * pr3;
            hsb = exp64(hsb);
            double kx = kn[1] + kn[2] * rt;
            double xnb = div64(1.0, 2.0 * (kn[3] + kn[4] * rt)) *
                         (-kn[1] - kn[2] * rt -
                          sqrt64(kx * kx - 4.0 * (kn[3] + kn[4] * rt) * (kn[5] + kn[6] * rt + kn[7] * log64(tf) - log64(pw))));
            double mnb = div64(55.51 * xnb, 1.0 - xnb);
            double hnb = qn[1] + qn[2] * tr2 + (qn[3] + qn[4] * tr + qn[5] * tr2 + qn[6] * tr3) * pr +
                         (qn[7] + qn[8] * tr + qn[9] * tr2) * pr2 + qn[10] * tr * pr3;
            hnb = exp64(hnb);
            double mnb2 = mnb * mnb, msb2 = msb * msb;
            a = div64(tt * hnb * mnb2 - tt * hsb * mnb * msb - 2.0 * mnb2 * msb + mnb * msb2 + hnb * mnb * msb * pn0 -
                          hsb * msb2 * pn0,
                      mnb2 - mnb * msb);
            b = div64(msb * (-(2.0 * tt * hnb * mnb) + tt * hsb * msb + mnb * msb - hnb * msb * pn0), mnb - msb);
            cq = div64(tt * hnb * mnb * msb2, mnb - msb);
            double a2 = a * a, a3 = a2 * a;
            double q = a2 - 3.0 * b;
            double q3 = q * q * q;
            double rr = -(2.0 * a3) + 9.0 * a * b - 27.0 * cq;
            double phi = atan(div64(sqrt64(fmax(4.0 * q3 - rr * rr, 0.)), rr));
            if (phi < 0.) phi = phi + PI;
            double msf = -(1.0 / 3.0 * (a + 2.0 * sqrt64(a2 - 3.0 * b) * cos(div64(PI + phi, 3.0))));
            msf = fmax(msf, 0.);
            double mnf = mnb * (1.0 - div64(msf, msb));
            mnf = fmax(mnf, 0.);
            double pn = div64(mnf, div64(hnb * mnf, mnf + msf) + div64(hsb * msf, mnf + msf));
            double wsf = div64(msf * 0.098076, 1.0 + msf * 0.098076 + mnf * 0.063012);
            double wnf = div64(mnf * 0.063012, 1.0 + msf * 0.098076 + mnf * 0.063012);
            ms = msf;
            ws = wsf;
            wn = wnf;
            parthno3l = 1.0 - div64(pn0 - pn, pn0);
            parthno3l = fmin(parthno3l, 1.);
        }
        ws = fmax(ws, 0.005);
    }
    // density F:4056-4070 (raw temperature)
    double dens;
    {
        const double* X = c_dens_x;
        double T = temp;
        double W = ws + wn;
        double WH = 1.0 - W;
        double T2 = T * T, T3 = T2 * T;
        double V1 = X[1] + X[2] * T + X[3] * T2 + X[4] * T3;
        double VS = X[5] + X[6] * T + X[7] * T2 + (X[8] + X[9] * T + X[10] * T2) * W +
                    (X[11] + X[12] * T + X[13] * T2) * W * W;
        double VN = X[14] + X[15] * T + X[16] * T2 + (X[17] + X[18] * T + X[19] * T2) * W +
                    (X[20] + X[21] * T + X[22] * T2) * W * W;
        double VMCAL = WH * (1. / 18.0160) * V1 + VS * ws * (1. / 98.080) + VN * wn * (1. / 63.0160);
        dens = div64(1.0, VMCAL) * 0.001;
    }
    // volume, radius, area, solubilities F:3068-3232
    double aw = 0., wt = 0., hhcl = 0., hhocl = 0., hhobr = 0., hclono2 = 0.;
    if (condliq == 1) {
        double vliq = div64(div64(ns * 98.076e-6, ws), dens);
        double rmode = cbrt(3.0 * vliq * (1. / (4. * PI * ndrop)) * AER_EXP_M45);
        rmean = rmode * AER_EXP_05;
        aliq = 4.0 * PI * (rmode * rmode) * ndrop * AER_EXP_2;
        double t = tl;
        const double rt = div64(1., t), rt2 = rt * rt, rt3 = rt2 * rt;
        double ph2o0 = exp64(18.452406985 - 3505.1578807 * rt - 330918.55082 * rt2 + 12725068.262 * rt3);
        aw = div64(pw * 1013., ph2o0);
        aw = fmin(aw, 1.);
        int br = (aw <= 0.05) ? 0 : ((aw < 0.85) ? 1 : 2);
        const double law = log64(aw);
        double y1 = c_an_a1[br] * exp64(c_an_b1[br] * law) + c_an_c1[br] * aw + c_an_d1[br];
        double y2 = c_an_a2[br] * exp64(c_an_b2[br] * law) + c_an_c2[br] * aw + c_an_d2[br];
        double m = y1 + (t - 190.) * (y2 - y1) * (1. / 70.);
        wt = div64(9800. * m, 98. * m + 1000.);
        wt = fmax(wt, 0.5);
        double mh2so4 = dens * wt * (1. / 9.8);
        double bigx = div64(wt, wt + (100. - wt) * 98. * (1. / 18.));
        hhcl = (0.094 - 0.61 * bigx + 1.2 * (bigx * bigx)) * exp64(-8.68 + (8515. - 10718. * exp64(0.7 * log64(bigx))) * rt);
        double qhcl = ck[12] * rhnm;
        double phcl0 = qhcl * ptot * (1. / 1013.0);
        double phcl1 = div64(div64(phcl0, r * t), div64(1., r * t) + div64(hhcl * ns, ms));
        A.parthcl = 1.0 - div64(phcl0 - phcl1, phcl0);
        double sclono2 = 0.306 + 24. * rt;
        hclono2 = 1.6e-6 * exp64(4710. * rt) * exp64(-sclono2 * mh2so4);
        double shocl = 0.0776 + 59.18 * rt;
        hhocl = 1.91e-6 * exp64(5862.4 * rt) * exp64(-shocl * mh2so4);
        hhobr = 4.6e-4 * exp64(4.5e3 * rt);
        // hhbr (F:3222-3228) feeds only the disabled HOCl+HBr branch of hetero
    }
    // total PSC area F:3240-3246, HNO3 partition F:3252-3258
    A.surf = aliq + anat * lnat + aice * lice;
    A.parthno3 = parthno3l * parthno3s;
    A.parthno3 = fmin(A.parthno3, 1.);
    // settling velocity F:3264-3348
    if (lice == 1 || lnat == 1) {
        const double rhoice = 0.928 * 1000.0, rhonat = 1.350 * 1000.0;
        double t = temp;
        double rpart = (lice * rice + lnat * rnatl) * 1.e-2;
        rpart = fmin(rpart, 535.e-6);
        if (rpart >= 0.5e-6) {
            double rhopart = lice * rhoice + lnat * rhonat;
            double rhoair = (hnm * 28.97 * (1. / 6.022e23)) * 1000.0;
            double tcel = t - 273.15;
            double netha = (1.718 + 0.0049 * tcel - 1.2e-5 * tcel * tcel) * 1.e-5;
            double rp3 = rpart * rpart * rpart;
            double cdnre2 = div64(32.0 * rp3 * (rhopart - rhoair) * rhoair * 9.80665, 3.0 * (netha * netha));
            double L = log64(cdnre2);
            double L2 = L * L, L3 = L2 * L, L4 = L2 * L2, L5 = L3 * L2, L6 = L3 * L3;
            double ynre = c_an_bnre[0] + c_an_bnre[1] * L + c_an_bnre[2] * L2 + c_an_bnre[3] * L3 +
                          c_an_bnre[4] * L4 + c_an_bnre[5] * L5 + c_an_bnre[6] * L6;
            double nre = exp64(ynre);
            if (nre >= 1.e-2) {
                A.vsed = div64(netha * nre, 2 * rhoair * rpart);
            } else {
                double lambda0 = 6.6e-8;
                double lambda = lambda0 * div64(1013.25, ptot) * (t * (1. / 293.15));
                double us = div64(2.0 * (rpart * rpart) * 9.80665 * (rhopart - rhoair), 9.0 * netha);
                double shapek = 1.2;
                A.vsed = div64(us, shapek) * (1.0 + div64(1.246 * lambda, rpart) +
                                              div64(0.42 * lambda, rpart) * exp64(-div64(0.87 * rpart, lambda)));
            }
        }
    }
    // ---------------- hetero F:3436-4026 ----------------
    double kl[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
    double ksl[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};  // K*S zero-initialised
    const double T = temp;
    const double rT = div64(1., T);
    if (condliq == 1) {
        double ZH2O = fmax(ck[2], 1.E-08 * hnm);
        double ZHCL = fmax(ck[12], 1.E-13 * hnm);
        double ZCLONO2 = fmax(ck[13], 1.E-13 * hnm);
        double ZHOBR = fmax(ck[25], 1.E-15 * hnm);
        const double rZH2O = div64(1., ZH2O), rZHCL = div64(1., ZHCL);
        const double pfac = rhnm * ptot * (1. / 1013.);
        double phcl = ZHCL * pfac;
        double pclono2 = ZCLONO2 * pfac;
        double phobr = ZHOBR * pfac;
        double wt2 = wt * wt, wt3 = wt2 * wt;
        double t0 = 144.11 + 0.166 * wt - 0.015 * wt2 + 2.18e-4 * wt3;
        double biga = 169.5 + 5.18 * wt - 0.0825 * wt2 + 3.27e-3 * wt3;
        double eta = biga * exp64(-1.43 * log64(T)) * exp64(div64(448., T - t0));
        const double Teta = div64(T, eta);
        double sqT = sqrt64(T);
        double ah = exp64(60.51 - 0.095 * wt + 0.0077 * wt2 - 1.61e-5 * wt3 - (1.76 + 2.52e-4 * wt2) * sqT +
                        div64(-805.89 + 253.05 * exp64(0.076 * log64(wt)), sqT));
        double dclono2 = 5.e-8 * Teta;
        double cclono2 = 1474. * sqT;
        double kh2o = 1.95e10 * exp64(-2800. * rT);
        double khh = 1.22e12 * exp64(-6200. * rT);
        double khydr = kh2o * aw + khh * ah * aw;
        double gbh2o = div64(4 * hclono2 * 0.082 * T * sqrt64(dclono2 * khydr), cclono2);
        double mhcl = hhcl * phcl;
        double khcl = 7.9e11 * ah * dclono2 * mhcl;
        double lclono2 = sqrt64(div64(dclono2, khydr + khcl));
        double fclono2 = div64(1., tanh(div64(rmean, lclono2))) - div64(lclono2, rmean);
        double grxn = fclono2 * gbh2o * sqrt64(1. + div64(khcl, khydr));
        double gbhcl = div64(grxn * khcl, khcl + khydr);
        double gs = 66.12 * hclono2 * mhcl * exp64(-1374. * rT);
        double fhcl = div64(1., 1 + div64(0.612 * (gs + gbhcl) * pclono2, phcl));
        double gps = fhcl * gs;
        double gbhclp = fhcl * gbhcl;
        double gb = gbhclp + div64(grxn * khydr, khcl + khydr);
        double gclono2 = div64(1., 1. + div64(1., gps + gb));
        double gclono2hcl = div64(gclono2 * (gps + gbhclp), gps + gb);
        double gclono2h2o = gclono2 - gclono2hcl;
        kl[0] = 0.25 * gclono2h2o * cclono2 * aliq * rZH2O;
        kl[1] = 0.25 * gclono2hcl * cclono2 * aliq * rZHCL;
        double chocl = 2009. * sqT;
        double dhocl = 6.4e-8 * Teta;
        double khoclhcl = 1.25e9 * ah * dhocl * mhcl;
        double lhocl = sqrt64(div64(dhocl, khoclhcl));
        double fhocl = div64(1., tanh(div64(rmean, lhocl))) - div64(lhocl, rmean);
        grxn = div64(4. * hhocl * 0.082 * T * sqrt64(dhocl * khoclhcl), chocl);
        double ghoclhcl = div64(1., 1. + div64(1., fhocl * grxn * fhcl));
        kl[4] = 0.25 * ghoclhcl * chocl * aliq * rZHCL;
        double mhobr = hhobr * phobr;
        double k2hobrhcl = exp64(0.542 * wt - 6.44e3 * rT + 10.3);
        double ratio = div64(mhobr, mhcl);
        if (ratio < 1.) {
            double k1hobrhcl = k2hobrhcl * mhcl;
            double dhobr = 6.2e-8 * Teta;
            double lhobr = sqrt64(div64(dhobr, k1hobrhcl));
            double fhobr = div64(1., tanh(div64(rmean, lhobr))) - div64(lhobr, rmean);
            double chobr = 1477. * sqT;
            double ghobrhcl = div64(4. * hhobr * 0.082 * T * sqrt64(dhobr * k1hobrhcl) * fhobr, chobr);
            kl[6] = 0.25 * ghobrhcl * chobr * aliq * rZHCL;
        } else {
            double k1hobrhcl = k2hobrhcl * mhobr;
            double dhcl = 7.8e-8 * Teta;
            double lhcl = sqrt64(div64(dhcl, k1hobrhcl));
            double fh = div64(1., tanh(div64(rmean, lhcl))) - div64(lhcl, rmean);
            double chcl = 2408. * sqT;
            double ghobrhcl = div64(4. * hhcl * 0.082 * T * sqrt64(dhcl * k1hobrhcl) * fh, chcl);
            kl[6] = div64(0.25 * ghobrhcl * chcl * aliq, ZHOBR);
        }
        double CBAR = 1400.1 * sqT;
        kl[2] = 0.25 * 0.1 * CBAR * aliq * rZH2O;
        double gxrn = exp64(29.24 - 0.396 * 100. * ws) + 0.114;
        double gbrno3h2o = div64(1., 1. / 0.805 + div64(1., gxrn));
        CBAR = 1221.4 * sqT;
        kl[5] = 0.25 * gbrno3h2o * CBAR * aliq * rZH2O;
    }
    if (lnat == 1) {
        double ZH2O = fmax(ck[2], 1.E-08 * hnm);
        double ZHCL = fmax(ck[12], 1.E-13 * hnm);
        const double PT = ptot * rT, NS = nnats, NL = nnatl;
        const double rZH2O = div64(1., ZH2O), rZHCL = div64(1., ZHCL);
#define NATR(G, M, RZ)                                                                                        \
    ((div64((G) * 4.56E4 * sqrt64(T * (1. / (M))) * (rnats * rnats) * NS, 1.0 + 3.3E4 * (G) * rnats * PT) +   \
      div64((G) * 4.56E4 * sqrt64(T * (1. / (M))) * (rnatl * rnatl) * NL, 1.0 + 3.3E4 * (G) * rnatl * PT)) * \
     (RZ))
        ksl[0] = NATR(0.004, 97.45, rZH2O);
        ksl[1] = NATR(0.2, 97.45, rZHCL);
        ksl[2] = NATR(4.0E-4, 108.0, rZH2O);
        ksl[5] = NATR(0., 142.0, rZH2O);
        ksl[3] = NATR(3.0E-3, 108.0, rZHCL);
        ksl[4] = NATR(0.1, 52.5, rZHCL);
        ksl[6] = NATR(0., 96.9, rZHCL);
#undef NATR
        ksl[7] = 0.;
    }
    if (lice == 1) {
        double ZH2O = fmax(ck[2], 1.E-08 * hnm);
        double ZHCL = fmax(ck[12], 1.E-13 * hnm);
        double ZHOBR = fmax(ck[25], 1.E-13 * hnm);
        const double PT = ptot * rT, NI = nice;
        const double rZH2O = div64(1., ZH2O), rZHCL = div64(1., ZHCL), rZHOBR = div64(1., ZHOBR);
#define ICER(G, M, RZ) \
    (div64((G) * 4.56E4 * sqrt64(T * (1. / (M))) * (rice * rice) * NI, 1.0 + 3.3E4 * (G) * rice * PT) * (RZ))
        ksl[1] = ICER(0.3, 97.45, rZHCL);
        ksl[0] = ICER(0.3, 97.45, rZH2O);
        ksl[2] = ICER(0.02, 108.0, rZH2O);
        ksl[3] = ICER(0.03, 108.0, rZHCL);
        ksl[4] = ICER(0.2, 52.5, rZHCL);
        ksl[5] = ICER(0.3, 142.0, rZH2O);
        ksl[6] = ICER(0.3, 96.9, rZHCL);
        ksl[7] = ICER(0.1, 96.9, rZHOBR);
#undef ICER
    }
    double f = (double)(lnat + lice);
#pragma unroll
    for (int m = 0; m < 8; m++) A.het[m] = kl[m] + f * ksl[m];
    A.het[8] = 0.;
}

// ----------------------------------------------------------------------------
// rate constants, F:920-1306
// ----------------------------------------------------------------------------
// Troe falloff: k0 = A0 T^E0, kinf = A1 T^E1, x = k0 n, k = x / (1 + x / kinf)
// 0.6^(1 / (1 + log10(x / kinf)^2)). Here k = x kinf / (kinf + x) (one
// division) and log10(x / kinf) = (ln A0 - ln A1 + ln n + (E0 - E1) ln T) / ln 10
// from the step's ln A (no logarithm per term).
__device__ __forceinline__ void cell_rates(const double* troe, const double* ltroe, double t, double hnm, double pm,
                                           double* K) {
    const double xln6 = LN06;
    double lntemp = log64(t);
    const double lnhnm = log64(hnm);
    const double rt = div64(1., t);  // Arrhenius exponents E / T as E * (1 / T)
    double ak0, ak1, rate, xpo, deq, l10, xk;
#define RK(name) K[K_##name]
#define TROE(I0, E0, I1, E1, OUT)                                                            \
    ak0 = troe[I0] * exp64(lntemp * (E0));                                                     \
    ak1 = troe[I1] * exp64(lntemp * (E1));                                                     \
    xk = ak0 * hnm;                                                                          \
    rate = div64(xk * ak1, ak1 + xk);                                                        \
    l10 = (ltroe[I0] - ltroe[I1] + lnhnm + lntemp * ((E0) - (E1))) * (1. / LN10);           \
    xpo = div64(1., 1. + l10 * l10);                                                         \
    OUT = rate * exp64(xln6 * xpo)
    TROE(0, -1.3, 1, 0.2, RK(a1));
    RK(a1et) = 1.63e-10 * exp64(60. * rt);
    RK(a2) = 1.4e-10 * exp64(-470. * rt);
    RK(a5) = 1.8e-11 * exp64(180. * rt);
    RK(a6) = 1.7e-12 * exp64(-940. * rt);
    RK(a6b) = 1.0e-14 * exp64(-490. * rt);
    double e200 = exp64(200. * rt);
    RK(a7) = 3.0e-11 * e200;
    double e250 = exp64(250. * rt);
    RK(a17) = 4.8e-11 * e250;
    RK(a19) = 2.8e-12 * exp64(-1800. * rt);
    double e270 = exp64(270. * rt);
    RK(a26) = 3.3e-12 * e270;
    RK(a27) = 1.5e-12 * exp64(19. * rt) + 2.1e-33 * exp64(920. * rt) * hnm;
    RK(a30) = 1.8e-12;
    RK(a31) = 1.8e-12;
    RK(a36) = 1.5e-13 * (1. + .6 * pm * (1. / 1013.));
    RK(b3) = 5.1e-12 * exp64(210. * rt);
    RK(b4) = 3.0e-12 * exp64((-1500. * rt));
    RK(b6) = 2.1e-11 * exp64((100. * rt));
    RK(b7) = 1.5e-11 * exp64((-3600. * rt));
    double em2450 = exp64((-2450. * rt));
    RK(b9) = 1.2e-13 * em2450;
    TROE(2, -4.4, 3, -0.7, RK(b12));
    TROE(4, -3.0, 5, 0.0, RK(b22));
    TROE(6, -3.4, 7, -1.1, RK(b23));
    deq = 2.1e-27 * exp64(10900. * rt);
    RK(b24) = div64(RK(b23), deq * hnm);
    double e460 = exp64(460. * rt);
    {
        double aux1 = 2.7e-17 * exp64(2199. * rt);
        double aux2 = 1. + div64(aux1, 6.5e-34 * exp64(1335. * rt) * hnm);
        RK(b27) = 2.4e-14 * e460 + div64(aux1, aux2);
    }
    RK(b28) = 1.3e-12 * exp64(380. * rt);
    deq = 2.7e-27 * exp64(11000. * rt);
    RK(b32) = div64(RK(b12), deq * hnm);
    double e20 = exp64(20. * rt);
    RK(b38) = 4.63e-11 * e20;
    RK(b39) = 7.25e-11 * e20;
    RK(c1a) = 1.31e-10;
    RK(c1b) = 0.35e-10;
    RK(c1c) = 0.09e-10;
    RK(c2) = 2.45e-12 * exp64((-1775. * rt));
    RK(c3) = 1.1e-10;
    TROE(16, -3.6, 17, 1.1, RK(c4));
    RK(c5) = 2.8e-12 * exp64((300. * rt));
    RK(c7) = 3.8e-13 * exp64((800. * rt));
    RK(c8) = 5.5e-12 * exp64(125. * rt);
    double em1600 = exp64((-1600. * rt));
    RK(c9) = 3.4e-11 * em1600;
    RK(c10) = 8.1e-11 * exp64((-30. * rt));
    RK(c12) = 5.2e-12;
    RK(c14) = 9.5e-14 * exp64((390. * rt));
    RK(c15) = 3.9e-14 * exp64((-900. * rt));
    RK(c17a) = 3.8e-12 * e200 * 0.7;
    RK(c17b) = 3.8e-12 * e200 * 0.3;
    RK(c18) = 3.3e-12 * exp64((-115. * rt));
    double em800 = exp64((-800. * rt));
    RK(c19) = 1.7e-11 * em800;
    RK(d2) = 2.3e-11 * exp64((-200. * rt));
    RK(d3) = 2.8e-11 * exp64(85. * rt);
    double e290 = exp64(290. * rt);
    RK(d4) = 6.4e-12 * e290;
    RK(d5) = 7.3e-12 * exp64((-1280. * rt));
    RK(d6) = 3.05e-11 * exp64((-2270. * rt));
    RK(d7) = 1.4e-11 * exp64(269. * rt);
    RK(d8) = 7.4e-12 * e270;
    double e230 = exp64(230. * rt);
    RK(d9) = 6.0e-13 * e230;
    RK(d10) = 3.6e-11 * exp64(-375. * rt);
    RK(d11) = 1.8e-12 * exp64((-250. * rt));
    TROE(8, -3.4, 9, -1.9, RK(d31));
    double em840 = exp64((-840. * rt));
    RK(d32) = 3.6e-12 * em840;
    RK(d33) = 2.6e-12 * e290;
    RK(d34) = 3.0e-12 * exp64((-500. * rt));
    RK(d35) = 1.7e-13;
    TROE(10, -2., 11, -1., RK(d36));
    RK(d37) = 3.4e-12 * exp64((-130. * rt));
    TROE(12, -4.5, 13, -2.0, RK(d60));
    deq = 1.72e-27 * exp64(8649. * rt);
    RK(d61) = div64(RK(d60), deq * hnm);
    RK(d62) = 1.0e-12 * exp64(-1590. * rt) + 3.0e-11 * em2450;
    RK(d90) = 2.3e-10;
    RK(d91) = 1.4e-10;
    RK(d92) = 2.0e-10;
    RK(d93) = 3.3e-10;
    RK(d94) = 1.64e-12 * exp64((-1520. * rt));
    RK(d95) = 2.4e-12 * exp64((-1250. * rt));
    RK(d96) = 1.0e-10;
    RK(d97) = 1.05e-12 * em1600;
    RK(e2) = 1.6e-11 * exp64((-780. * rt));
    RK(e3) = 1.9e-11 * e230;
    double e260 = exp64(260. * rt);
    RK(e4) = 8.8e-12 * e260;
    RK(e5a) = 9.5e-13 * exp64(550. * rt);
    RK(e5b) = 2.3e-12 * e260;
    RK(e5c) = 4.1e-13 * e290;
    RK(e6) = 1.5e-12 * e230;
    RK(e7) = 4.8e-12 * exp64(-310. * rt);
    RK(e8) = 1.9e-11 * exp64(215. * rt);
    RK(e9) = 1.5e-10;
    RK(e10) = 1.7e-11 * e250;
    RK(e11) = 5.5e-12 * e200;
    TROE(14, -3.2, 15, -2.9, RK(e13));
    RK(e15) = 4.5e-12 * e460;
    RK(e16) = 1.2e-10 * exp64((-430. * rt));
    RK(e50) = 1.8e-10;
    RK(e51) = 2.35e-12 * exp64((-1300. * rt));
    RK(e52) = 1.5e-10;
    RK(e53) = 1.0e-10;
    RK(e54) = 2.0e-12 * em840;
    RK(hk1) = 4.23e-28 * hnm * (rt * rt);
    RK(hk2) = 6.0e-34 * exp64(2.4 * log64(300. * rt)) * hnm;
    RK(hk3) = 8.e-12 * exp64((-2060. * rt));
    RK(hk4) = 2.15e-11 * exp64(110. * rt);
    RK(hk5) = 3.3e-11 * exp64(55. * rt);
#undef TROE
#undef RK
}

// fixed per-cell quantities of the iteration
template <typename T>
struct CellFixT {
    T o2, n2, h2, co2, hnm;
    T parthno3, parth2o, parthcl, parthbr;
    T rain_hno3, rain_hno4, rain_hcl, rain_hbr, rain_h2o2, rain_ch2o, rain_ch3o2h;
    T sza;
};
using CellFix = CellFixT<double>;

// ----------------------------------------------------------------------------
// one pass of the iteration, F:1350-2372; ck (43), cc (15), ck0 (42)
// ----------------------------------------------------------------------------
// T = double: the reference's arithmetic (every call of the FP64 path);
// T = float: the same statements in FP32, for the start of the mixed solver.
// Its quotients (pass_div): the IEEE division in FP64 (the reference's
// arithmetic); in FP32 (the start only seeds Newton) the fast division,
// within 2 ulp for divisors below 2^126
template <typename T>
__device__ __forceinline__ T pass_div(T a, T b) {
    return a / b;
}
template <>
__device__ __forceinline__ float pass_div<float>(float a, float b) {
    return __fdividef(a, b);
}

template <typename T>
__device__ __forceinline__ void cell_pass(const CellFixT<T>& F, const T* __restrict__ K, const T* __restrict__ tj,
                                          const T* __restrict__ het, const T* __restrict__ ck0, T dt, T* ck,
                                          T* cc) {
    const T a3et = T(1.2e-10), a23a = T(7.2e-11), a23b = T(6.9e-12), a23c = T(1.6e-12);
#define KK(name) K[K_##name]
#define PDIV(a, b) pass_div<T>(a, b)
#define CK(m) ck[(m)-1]
#define CC(m) cc[(m)-1]
#define TJ(name) tj[J_##name]
#define HET(m) het[(m)-1]
    const T o2 = F.o2, n2 = F.n2, h2 = F.h2, hnm = F.hnm, co2 = F.co2;
    const T parthno3 = F.parthno3, parth2o = F.parth2o, parthcl = F.parthcl, parthbr = F.parthbr;
    T a, b, day, ch3o, hco;
    if (F.sza <= T(95.)) {
        day = T(1.);
        CC(15) = PDIV(((KK(c2) * CC(2) + KK(c1a) * CC(1) + KK(d5) * CC(3)) * CK(2)), (KK(c4) * o2 + KK(c3) * CC(4)));
        ch3o = PDIV((KK(c1b) * CC(1) * CK(2) + (KK(c5) * CC(8) + T(2.) * KK(c14) * CK(29) + KK(c18) * CC(11)) * CK(29) +
                     TJ(ch3o2h) * CK(30)),
                    (KK(c15) * o2));
        hco = PDIV((KK(c8) * CC(2) + KK(c9) * CC(4) + KK(c10) * CC(3) + KK(c19) * CC(9) + TJ(ch2o_hco)) * CK(28),
                   (KK(c12) * o2));
        T r1 = PDIV((TJ(o3_o1d) + TJ(o3_o3p) + KK(a2) * CC(14) + KK(a6) * CC(2) + KK(a6b) * CC(6) + KK(b4) * CC(8) +
                      KK(d2) * CC(3)),
                     (KK(hk2) * o2));
        T r2 = PDIV(T(1.), (T(1.) + r1));
        CC(5) = r2 * CK(8);
        CC(4) = r1 * CC(5);
        T r3 = PDIV(TJ(o3_o1d), (KK(hk4) * n2 + KK(hk5) * o2));
        CC(1) = r3 * CC(5);
        T r4 = PDIV((KK(a5) * CC(4) + KK(a36) * CK(9) + KK(a19) * h2),
                    (KK(a1) * o2 + KK(a2) * CC(5) + (a23a + a23b + a23c) * CC(6)));
        CC(14) = r4 * CC(2);
        T r7 = PDIV(TJ(no), (KK(b7) * o2 + KK(b6) * CC(8)));
        T r8 = PDIV((KK(b9) * CC(5)), (TJ(no3_no) + TJ(no3_no2) + KK(b12) * CC(7)));
        T r5 = PDIV((TJ(no2) + KK(b3) * CC(4) + TJ(no3_no) * r8),
                    (KK(b4) * CC(5) + KK(a26) * CC(6) + KK(d4) * CC(11) + KK(e4) * CC(12) + KK(c5) * CK(29)));
        CC(7) = PDIV(CK(21), (T(1.) + r5 + r7 * r5 + r8));
        CC(8) = r5 * CC(7);
        CC(10) = r7 * CC(8);
        CC(13) = r8 * CC(7);
        T r6 = PDIV((KK(a6) * CC(5) + KK(a30) * CK(17) + KK(c8) * CK(28) + KK(d8) * CC(11) + KK(e10) * CC(12) +
                      KK(a1) * o2 * r4),
                     ((a23a + a23b + a23c) * CC(14) + KK(a6b) * CC(5) + KK(a7) * CC(4) + KK(a26) * CC(8) +
                      T(2.) * KK(a27) * CC(6) + KK(a17) * CC(2) + KK(d7) * CC(3) + KK(d10) * CC(3) + KK(d33) * CC(11) +
                      KK(e7) * CC(9) + KK(e15) * CC(12)));
        a = T(.5);
        b = T(1.) - a;
        CC(6) = a * CC(6) + b * CC(2) * r6;
        T r13 = PDIV(KK(d31) * CC(7),
                     (TJ(clono2_cl) + TJ(clono2_clo) + KK(d32) * CC(4) + HET(1) * CK(3) + HET(2) * CK(13)));
        T r9 = PDIV((KK(d33) * CC(6) + HET(1) * CK(3) * r13), (HET(5) * CK(13) + KK(d35) * CC(4) + TJ(hocl)));
        T r10 = PDIV((KK(d60) * CC(11)), (KK(d61) * hnm + TJ(cl2o2)));
        T r12 = PDIV(KK(e5c) * CC(12), TJ(brcl));
        T r11 = PDIV((KK(d3) * CC(4) + KK(d4) * CC(8) + KK(d8) * CC(2) + KK(c18) * CK(29) + KK(e5b) * CC(12) +
                       TJ(clono2_cl) * r13 + TJ(hocl) * r9 + T(2.) * TJ(cl2o2) * r10 + TJ(brcl) * r12),
                      (KK(d2) * CC(5) + KK(d5) * CK(2) + KK(d7) * CC(6) + KK(d10) * CC(6) + KK(d37) * CK(15)));
        CC(11) = a * CC(11) + PDIV(b * CK(23), (T(1.) + r11));
        CC(3) = r11 * CC(11);
        T r27 = PDIV(KK(e13) * CC(7), (TJ(brono2) + KK(e8) * CC(4)));
        T r28 = PDIV(KK(e15) * CC(6), (TJ(hobr) + KK(e16) * CC(4)));
        T r29 = PDIV(KK(e5c) * CC(11), TJ(brcl));
        T r30 = PDIV((KK(e3) * CC(4) + KK(e4) * CC(8) + KK(e5a) * CC(11) + KK(e5b) * CC(11) + T(2.) * KK(e6) * CC(12) +
                       KK(e10) * CC(2) + TJ(bro) + TJ(brono2) * T(0.85) * r27 + TJ(hobr) * r28 + TJ(brcl) * r29),
                      (KK(e2) * CC(5) + KK(e7) * CC(6) + KK(c19) * CK(28)));
        CC(12) = a * CC(12) + PDIV(b * CK(24), (T(1.) + r30));
        CC(9) = r30 * CC(12);
        T coea = T(2.) * KK(a31) + T(2.) * (KK(a17) + KK(a27) * r6 + (a23b + a23c) * r4) * r6;
        T coeb = KK(b27) * CK(5) * parthno3 + KK(b22) * CC(7) + KK(b28) * CK(22) + KK(b23) * CC(7) * r6 +
                      KK(c2) * CK(2) + KK(c7) * CK(29) * r6 + KK(c8) * CK(28) + KK(c17a) * CK(30) +
                      KK(d7) * CC(3) * r6 + KK(d9) * CC(11) + KK(d11) * CK(13) * parthcl + KK(d33) * CC(11) * r6 +
                      KK(d34) * CK(15) + KK(e11) * CK(19) * parthbr + KK(e7) * CC(9) * r6 + KK(e15) * CC(12) * r6;
        T t01 = T(2.) * (KK(a1et) * CC(1) + TJ(h2o)) * CK(3) * parth2o;
        T t02 = ((KK(c1a) + KK(c1b)) * CK(2) + T(2.) * a3et * h2) * CC(1);
        T t03 = KK(c3) * CC(15) * CC(4);
        T t04 = TJ(ch3o2h) * CK(30);
        T t05 = KK(c15) * ch3o * o2;
        T t06 = (TJ(ch2o_hco) + KK(c9) * CC(4)) * CK(28);
        T t07 = KK(c12) * hco * o2;
        T t08 = TJ(hno3) * CK(5) * parthno3;
        T t09 = (KK(b24) * hnm + TJ(hno4)) * CK(22);
        T t10 = (KK(d35) * CC(4) + KK(d37) * CC(3) + TJ(hocl)) * CK(15);
        T t11 = T(2.) * TJ(h2o2) * CK(17);
        T t12 = KK(d6) * h2 * CC(3);
        T t13 = TJ(hobr) * CK(26);
        T t14 = KK(e16) * CC(4) * CK(26);
        T t15 = TJ(hbr) * CK(19);
        T coec = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13 + t14 + t15;
        T argum = coeb * coeb + T(4.) * coea * coec;
        argum = fmax(argum, T(0.));
        CC(2) = a * CC(2) + PDIV(b * (sqrt(argum) - coeb), (T(2.) * coea));
    } else {
        day = T(0.);
        CC(14) = T(0.);
        CC(15) = T(0.);
        ch3o = T(0.);
        hco = T(0.);
        CC(1) = T(0.);
        CC(4) = T(0.);
        CC(5) = CK(8);
        CC(2) = T(0.);
        CC(3) = T(0.);
        CC(6) = T(0.);
        CC(8) = T(0.);
        T r8 = PDIV(KK(b9) * CC(5), (KK(b12) * fmax(CC(7), T(1.e-30))));
        CC(7) = PDIV(CK(21), (T(1.) + r8));
        CC(13) = r8 * CC(7);
        CC(10) = T(0.);
        CC(11) = fmax(CK(23), T(0.));
        CC(9) = T(0.);
        CC(12) = fmax(CK(24), T(0.));
    }
    // production / loss, F:1758-2358; update F:2364-2372 applied per species
    const T rain_hno3 = F.rain_hno3, rain_hno4 = F.rain_hno4, rain_hcl = F.rain_hcl, rain_hbr = F.rain_hbr,
                 rain_h2o2 = F.rain_h2o2, rain_ch2o = F.rain_ch2o, rain_ch3o2h = F.rain_ch3o2h;
    T pr[NBCON - 1], pe[NBCON - 1];
#define PR(m) pr[(m)-1]
#define PE(m) pe[(m)-1]
    T t01, t02, t03, t04, t05, t06, t07, t08, t09, t10, t11, t12, t13, t14;
    PR(1) = T(0.e0);
    PE(1) = TJ(n2o) + (KK(b38) + KK(b39)) * CC(1);
    PR(2) = T(0.e0);
    PE(2) = KK(c2) * CC(2) + KK(c1a) * CC(1) + KK(c1b) * CC(1) + KK(c1c) * CC(1) + KK(d5) * CC(3);
    PR(3) = KK(c2) * CC(2) * CK(2) + KK(c8) * CC(2) * CK(28) + KK(c17a) * CK(30) * CC(2) +
            KK(c17b) * CK(30) * CC(2) + (KK(a17) * CC(2) + a23c * CC(14)) * CC(6) + KK(a19) * CC(2) * h2 +
            KK(a30) * CC(2) * CK(17) + KK(a31) * CC(2) * CC(2) + KK(b27) * CC(2) * CK(5) * parthno3 +
            KK(d11) * CC(2) * CK(13) * parthcl;
    PE(3) = (TJ(h2o) + KK(a1et) * CC(1)) * parth2o;
    PR(4) = T(2.) * KK(b39) * CC(1) * CK(1);
    PE(4) = T(2.) * KK(b6) * CC(10) * CC(8) + rain_hno3 * CK(5) + rain_hno4 * CK(22);
    PE(4) = PDIV(PE(4), CK(4));
    PR(5) = KK(b22) * CC(2) * CC(7) + HET(1) * CK(14) * CK(3) + HET(2) * CK(14) * CK(13) +
            T(2.) * HET(3) * CK(6) * CK(3) + HET(4) * CK(6) * CK(13) + HET(6) * CK(20) * CK(3);
    PE(5) = (TJ(hno3) + KK(b27) * CC(2)) * parthno3 + rain_hno3;
    PR(6) = KK(b12) * CC(13) * CC(7);
    PE(6) = TJ(n2o5) + KK(b32) * hnm + HET(3) * CK(3) + HET(4) * CK(13);
    PR(7) = T(3.) * (TJ(cfc11) + KK(d90) * CC(1)) * CK(31) + T(2.) * (TJ(cfc12) + KK(d91) * CC(1)) * CK(32) +
            T(3.) * (TJ(cfc113) + KK(d92) * CC(1)) * CK(33) + T(4.) * (TJ(ccl4) + KK(d93) * CC(1)) * CK(34) +
            T(3.) * (TJ(ch3ccl3) + KK(d94) * CC(2)) * CK(35) + T(1.) * (TJ(ch3cl) + KK(d95) * CC(2)) * CK(36) +
            T(1.) * (TJ(hcfc22) + KK(d96) * CC(1) + KK(d97) * CC(2)) * CK(37) +
            T(1.) * (TJ(h1211) + KK(e52) * CC(1)) * CK(39);
    PE(7) = rain_hcl * CK(13);
    PE(7) = PDIV(PE(7), CK(7));
    T ratio = PDIV(TJ(cl2o2), (TJ(cl2o2) + KK(d61) * hnm));
    PR(8) = T(2.) * TJ(o2) * o2 + KK(a26) * CC(6) * CC(8) + KK(c5) * CC(8) * CK(29);
    t01 = T(2.) * KK(hk1) * CC(4) * CC(4);
    t02 = T(2.) * KK(hk3) * CC(5) * CC(4);
    t03 = T(2.) * KK(b3) * CC(7) * CC(4);
    t04 = T(2.) * KK(d3) * CC(11) * CC(4);
    t05 = T(2.) * KK(d60) * ratio * CC(11) * CC(11);
    t06 = fmin(TJ(hocl) * CK(15), KK(d33) * CC(6) * CC(11));
    t07 = T(2.) * fmin(KK(e5c) * CC(12) * CC(11), TJ(brcl) * CK(27));
    t08 = T(2.) * KK(e5b) * CC(12) * CC(11) * day;
    t09 = fmin(KK(e15) * CC(12) * CC(6), TJ(hobr) * CK(26));
    t10 = T(2.) * KK(e6) * CC(12) * CC(12) * day;
    t11 = T(2.) * PDIV(TJ(no3_no), fmax(TJ(no3_no) + TJ(no3_no2), T(1.e-30))) * TJ(clono2_cl) * CK(14);
    t12 = (KK(a2) * CC(14) + KK(a6) * CC(2) + KK(a6b) * CC(6)) * CC(5) + (KK(a5) * CC(2) + KK(a7) * CC(6)) * CC(4);
    t13 = PDIV(T(2.) * KK(b9) * CC(7) * CC(5) * TJ(no3_no), fmax(TJ(no3_no) + TJ(no3_no2), T(1.e-30)));
    PE(8) = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13;
    PE(8) = PDIV(PE(8), CK(8));
    PR(9) = TJ(co2) * co2 + TJ(ch2o_co) * CK(28) + KK(c12) * hco * o2;
    PE(9) = KK(a36) * CC(2);
    PR(10) = KK(e5a) * CC(12) * CC(11);
    PE(10) = TJ(oclo);
    PR(11) = T(0.);
    PE(11) = T(0.);
    PR(12) = T(0.);
    PE(12) = T(0.);
    PR(13) = (KK(c10) * CK(28) + KK(d5) * CK(2) + KK(d7) * CC(6) + KK(d6) * h2) * CC(3) + KK(d9) * CC(2) * CC(11);
    PE(13) = (TJ(hcl) + KK(d11) * CC(2)) * parthcl + HET(2) * CK(14) + HET(4) * CK(6) + HET(5) * CK(15) +
             HET(7) * CK(26) + rain_hcl;
    PR(14) = KK(d31) * CC(7) * CC(11);
    PE(14) = TJ(clono2_cl) + TJ(clono2_clo) + KK(d32) * CC(4) + HET(1) * CK(3) + HET(2) * CK(13);
    PR(15) = KK(d33) * CC(6) * CC(11) + HET(1) * CK(14) * CK(3);
    PE(15) = TJ(hocl) + KK(d34) * CC(2) + KK(d35) * CC(4) + KK(d37) * CC(3) + HET(5) * CK(13) + HET(9) * CK(19);
    PR(16) = KK(d37) * CK(15) * CC(3) + KK(d62) * CC(11) * CC(11) + HET(2) * CK(14) * CK(13) +
             HET(5) * CK(15) * CK(13);
    PE(16) = TJ(cl2);
    PR(17) = KK(a27) * CC(6) * CC(6);
    PE(17) = TJ(h2o2) + KK(a30) * CC(2) + rain_h2o2;
    PR(18) = KK(d36) * CC(3) * CC(7) + HET(4) * CK(6) * CK(13);
    PE(18) = TJ(clno2);
    PR(19) = KK(e7) * CC(6) * CC(9) + KK(c19) * CK(28) * CC(9);
    PE(19) = (KK(e11) * CC(2) + KK(e9) * CC(1) + TJ(hbr)) * parthbr + HET(8) * CK(26) + HET(9) * CK(15) + rain_hbr;
    PR(20) = KK(e13) * CC(12) * CC(7);
    PE(20) = TJ(brono2) + KK(e8) * CC(4) + HET(6) * CK(3);
    PR(21) = (TJ(hno4) + KK(b28) * CC(2) + KK(b24) * hnm) * CK(22) + TJ(hno3) * CK(5) * parthno3 +
             T(2.) * (TJ(n2o5) + KK(b32) * hnm) * CK(6) + T(2.) * KK(b39) * CC(1) * CK(1) + TJ(clno2) * CK(18) +
             KK(b27) * CK(5) * parthno3 * CC(2) + KK(d32) * CK(14) * CC(4) +
             (TJ(clono2_cl) + TJ(clono2_clo)) * CK(14) + TJ(brono2) * CK(20) + KK(e8) * CK(20) * CC(4);
    PE(21) = (KK(d31) * CC(11) + KK(b22) * CC(2) + KK(b23) * CC(6) + T(2.) * KK(b12) * CC(13) + KK(d36) * CC(3) +
              KK(e13) * CC(12)) *
                 CC(7) +
             T(2.) * KK(b6) * CC(10) * CC(8);
    PE(21) = PDIV(PE(21), CK(21));
    PR(22) = KK(b23) * CC(6) * CC(7);
    PE(22) = TJ(hno4) + KK(b28) * CC(2) + KK(b24) * hnm + rain_hno4;
    t01 = T(2.) * (KK(d61) * hnm + TJ(cl2o2)) * CK(25);
    t02 = (TJ(clono2_cl) + TJ(clono2_clo) + KK(d32) * CC(4)) * CK(14);
    t03 = (TJ(hocl) + KK(d34) * CC(2) + KK(d35) * CC(4)) * CK(15);
    t04 = TJ(oclo) * CK(10) + (TJ(hcl) + KK(d11) * CC(2)) * CK(13) * parthcl;
    t05 = T(2.) * TJ(cl2) * CK(16);
    t06 = TJ(clno2) * CK(18);
    t07 = TJ(brcl) * CK(27);
    t08 = T(3.) * (TJ(cfc11) + KK(d90) * CC(1)) * CK(31);
    t09 = T(2.) * (TJ(cfc12) + KK(d91) * CC(1)) * CK(32);
    t10 = T(3.) * (TJ(cfc113) + KK(d92) * CC(1)) * CK(33);
    t11 = T(4.) * (TJ(ccl4) + KK(d93) * CC(1)) * CK(34);
    t12 = T(3.) * (TJ(ch3ccl3) + KK(d94) * CC(2)) * CK(35);
    t13 = T(1.) * (TJ(ch3cl) + KK(d95) * CC(2)) * CK(36);
    t14 = T(1.) * (TJ(hcfc22) + KK(d96) * CC(1) + KK(d97) * CC(2)) * CK(37);
    PR(23) = t01 + t02 + t03 + t04 + t05 + t06 + t07 + t08 + t09 + t10 + t11 + t12 + t13 + t14;
    PE(23) = (KK(d31) * CC(7) + T(2.) * KK(d60) * CC(11) + T(2.) * KK(d62) * CC(11) + KK(e5a) * CC(12) +
              KK(e5c) * CC(12) + KK(d9) * CC(2) + KK(d33) * CC(6)) *
                 CC(11) +
             (KK(c10) * CK(28) + KK(d5) * CK(2) + KK(d7) * CC(6) + KK(d6) * h2 + KK(d36) * CC(7) +
              KK(d37) * CK(15)) *
                 CC(3);
    PE(23) = PDIV(PE(23), CK(23));
    PR(24) = TJ(hobr) * CK(26) + TJ(brono2) * CK(20) + KK(e8) * CK(20) * CC(4) + KK(e16) * CK(26) * CC(4) +
             TJ(brcl) * CK(27) + (KK(e11) * CC(2) + KK(e9) * CC(1) + TJ(hbr)) * CK(19) * parthbr +
             T(2.) * HET(8) * CK(19) * CK(26);
    PE(24) = (KK(e13) * CC(7) + KK(e5c) * CC(11) + KK(e15) * CC(6)) * CC(12) + KK(c19) * CC(9) * CK(28) +
             KK(e7) * CC(9) * CC(6);
    PE(24) = PDIV(PE(24), CK(24));
    PR(25) = KK(d60) * CC(11) * CC(11);
    PE(25) = TJ(cl2o2) + KK(d61) * hnm;
    PR(26) = KK(e15) * CC(12) * CC(6) + HET(6) * CK(20) * CK(3);
    PE(26) = TJ(hobr) + KK(e16) * CC(4) + HET(7) * CK(13) + HET(8) * CK(19);
    PR(27) = KK(e5c) * CC(11) * CC(12) + HET(7) * CK(26) * CK(13) + HET(9) * CK(19) * CK(15);
    PE(27) = TJ(brcl);
    PR(28) = (KK(c1c) * CC(1) * CK(2) + KK(c3) * CC(4) * CC(15) + KK(c15) * ch3o * o2 + KK(c17b) * CC(2) * CK(30));
    PE(28) = KK(c8) * CC(2) + KK(c9) * CC(4) + KK(c10) * CC(3) + KK(c19) * CC(9) + TJ(ch2o_hco) + TJ(ch2o_co) +
             rain_ch2o;
    PR(29) = KK(c4) * CC(15) * o2 + KK(c17a) * CC(2) * CK(30);
    PE(29) = T(2.) * KK(c14) * CK(29) + KK(c7) * CC(6) + KK(c5) * CC(8) + KK(c18) * CC(11);
    PR(30) = KK(c7) * CK(29) * CC(6);
    PE(30) = KK(c17a) * CC(2) + KK(c17b) * CC(2) + TJ(ch3o2h) + rain_ch3o2h;
    PR(31) = T(0.);
    PE(31) = TJ(cfc11) + KK(d90) * CC(1);
    PR(32) = T(0.);
    PE(32) = TJ(cfc12) + KK(d91) * CC(1);
    PR(33) = T(0.);
    PE(33) = TJ(cfc113) + KK(d92) * CC(1);
    PR(34) = T(0.);
    PE(34) = TJ(ccl4) + KK(d93) * CC(1);
    PR(35) = T(0.);
    PE(35) = TJ(ch3ccl3) + KK(d94) * CC(2);
    PR(36) = T(0.);
    PE(36) = TJ(ch3cl) + KK(d95) * CC(2);
    PR(37) = T(0.);
    PE(37) = TJ(hcfc22) + KK(d96) * CC(1) + KK(d97) * CC(2);
    PR(38) = T(0.);
    PE(38) = TJ(ch3br) + KK(e50) * CC(1) + KK(e51) * CC(2);
    PR(39) = T(0.);
    PE(39) = TJ(h1211) + KK(e52) * CC(1);
    PR(40) = T(0.);
    PE(40) = TJ(h1301) + KK(e53) * CC(1);
    PR(41) = (TJ(ch3br) + KK(e50) * CC(1) + KK(e51) * CC(2)) * CK(38) + (TJ(h1211) + KK(e52) * CC(1)) * CK(39) +
             (TJ(h1301) + KK(e53) * CC(1)) * CK(40) + T(2.) * (KK(e54) * CC(2) + TJ(ch2br2)) * CK(42);
    PE(41) = rain_hbr * CK(19);
    PE(41) = PDIV(PE(41), CK(41));
    PR(42) = T(0.);
    PE(42) = TJ(ch2br2) + KK(e54) * CC(2);
#pragma unroll
    for (int m = 0; m < NBCON - 1; m++) ck[m] = PDIV((ck0[m] + dt * pr[m]), (T(1.) + dt * pe[m]));
#undef PR
#undef PE
#undef KK
#undef PDIV
#undef CK
#undef CC
#undef TJ
#undef HET
}

// ----------------------------------------------------------------------------
// conserv, F:2539-2613, on the written-back mixing ratios of one cell
// q: 43 mixing ratios, h: 15 mixing ratios
// ----------------------------------------------------------------------------
__device__ __forceinline__ void cell_conserv(double* q, double* h) {
#define Q(m) q[(m)-1]
#define H(m) h[(m)-1]
    double totmas = Q(10) + Q(13) + Q(14) + Q(15) + 2. * Q(16) + Q(18) + Q(23) + 2. * Q(25);
    double rapcly = div64(Q(7) - Q(27), totmas);
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
    double rapnoy = div64(fmax((Q(4) - Q(14) - Q(18) - Q(20)), 0.), totmas);
    H(7) = H(7) * rapnoy;
    H(8) = H(8) * rapnoy;
    H(10) = H(10) * rapnoy;
    H(13) = H(13) * rapnoy;
    Q(5) = Q(5) * rapnoy;
    Q(6) = Q(6) * rapnoy;
    Q(21) = Q(21) * rapnoy;
    Q(22) = Q(22) * rapnoy;
    totmas = Q(19) + Q(20) + Q(24) + Q(26) + Q(27);
    double rapbry = div64(Q(41), totmas);
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

}  // namespace rpb
