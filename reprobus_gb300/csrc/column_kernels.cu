// column_kernels.cu — the per-column physics that the time loop runs around the
// chemistry step, on the GPU, over the reference's FP64 Fortran-layout arrays:
//
//   k_sediment    sedimentation of H2O, NOy and HNO3      F:2416-2522 (called :420)
//   k_forcing     tropospheric relaxation tropo            F:4077-4574 (called :373)
//                 CO relaxation co_tropo                   F:4577-4639 (called :377)
//                 tropospheric H2O ecmwfh2o                F:8621-8658 (called :382)
//   k_geo_levels  pressure, virtual temperature and geopotential
//                 increments of the regular grid            altitude.f90:32-57
//   k_geo_sum     the hypsometric sum up each regular column altitude.f90:51-57
//   k_altitude    geometric altitude of every trajectory    altitude.f90:59-146
//   k_swap64      big-endian FP64 of the history record    F:231-235, F:587-588
//
// (F = src/reprobus_l137_20230723.f.) All of them are HBM-bound byte moves
// with a few transcendentals per cell; the columns are independent, so each
// kernel takes a column (a vertical recurrence) or a cell per thread, with
// consecutive threads on consecutive longitudes (coalesced planes). The
// sedimentation and geopotential recurrences keep the reference's evaluation
// order and round every operation separately (__d*_rn, no FMA contraction).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/reprobus_chem.h"
#include "handle_info.h"
#include "tropo_tables.h"

extern "C" int reprobus_set_error(int code, const char* fmt, ...);

using namespace rpb;

#define COL_TRY(x)                                                                                              \
    do {                                                                                                        \
        cudaError_t e_ = (x);                                                                                   \
        if (e_ != cudaSuccess)                                                                                  \
            return reprobus_set_error(REPROBUS_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, \
                                      __LINE__);                                                                \
    } while (0)

namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// ---------------------------------------------------------------------------
// sedimentation, F:2416-2522
// ---------------------------------------------------------------------------
struct SedArgs {
    const double* pre;  // trajpre(:,:,:,irapp)
    const double* tem;  // trajtem(:,:,:,irapp)
    double* qj1;
    const double* vsed;  // vsed3d(nlon,nlat,nivbas)
    const double* ph2o;  // parth2osed
    const double* pno3;  // parthno3sed
    int nlon, nlat, niv, nivbas, nivhau, nivh2o, row0, nrows;
    double dt;
};

// q(k) + q_up (1 - part_up) hnm_up / hnm fracup - q_self (1 - part) fracdown,
// left to right as F:2470-2476 writes it
__device__ __forceinline__ double sed_update(double q, double q_up, double part_up, double hnm_up, double hnm,
                                             double fracup, double q_self, double part, double fracdown) {
    const double gain = mul(dvd(mul(mul(q_up, sub(1.0, part_up)), hnm_up), hnm), fracup);
    return sub(add(q, gain), mul(mul(q_self, sub(1.0, part)), fracdown));
}

// Both of the reference's loops read only values from before the loop (level
// iniv-1 is updated after level iniv), so every level of a column can be
// updated at once from the old values. A block owns SED_COLS whole columns
// (consecutive longitudes: each level plane is read coalesced) with
// SED_LANES threads per column, each on every SED_LANES-th level: all threads
// compute their new values from the old ones, meet at one block barrier (no
// other block touches these columns), then store them.
constexpr int SED_COLS = 32, SED_LANES = 16, SED_KMAX = 8;  // levels nivhau..nivbas <= SED_LANES * SED_KMAX

__global__ void __launch_bounds__(SED_COLS * SED_LANES) k_sediment(SedArgs A) {
    const int t = blockIdx.x * SED_COLS + threadIdx.x;
    const bool live = t < A.nlon * A.nrows;
    const size_t col = live ? (size_t)(t % A.nlon) + (size_t)A.nlon * (A.row0 + t / A.nlon) : 0;
    const size_t pl = (size_t)A.nlon * A.nlat;
    const size_t p3 = pl * A.niv;  // one species of qj1
    double* q3 = A.qj1 + 2 * p3;   // H2O
    double* q4 = A.qj1 + 3 * p3;   // NOy
    double* q5 = A.qj1 + 4 * p3;   // HNO3
    // hnm of F:2443-2446 (the constant cancels in hnm_up / hnm)
    auto hnm_at = [&](size_t i) { return dvd(A.pre[i], mul(A.tem[i], 1.38e-19)); };
    double n3[SED_KMAX], n4[SED_KMAX], n5[SED_KMAX];
#pragma unroll
    for (int j = 0; j < SED_KMAX; j++) {
        const int k = A.nivhau + (int)threadIdx.y + j * SED_LANES;  // 1-based level
        if (!live || k > A.nivbas) continue;
        const size_t i = col + pl * (size_t)(k - 1), iu = i - pl;
        const double p = A.pre[i], p_up = A.pre[iu];
        const double h = hnm_at(i), h_up = hnm_at(iu);
        const double v = A.vsed[i], v_up = A.vsed[iu];
        const double dz = mul(7000., log(dvd(p, p_up)));
        const double fu = fmin(dvd(mul(v_up, A.dt), dz), 1.0);
        const double fd = fmin(dvd(mul(v, A.dt), dz), 1.0);
        // H2O, levels nivh2o-1 .. nivhau (F:2456-2480)
        if (k <= A.nivh2o - 1) {
            const double q = q3[i];
            n3[j] = sed_update(q, q3[iu], A.ph2o[iu], h_up, h, fu, q, A.ph2o[i], fd);
        }
        // NOy and HNO3, levels nivbas .. nivhau (F:2482-2514; the NOy update
        // moves the HNO3 flux, the 01/12/2012 fix at :2493)
        const double q = q5[i], q_up = q5[iu], s = A.pno3[i], s_up = A.pno3[iu];
        n4[j] = sed_update(q4[i], q_up, s_up, h_up, h, fu, q, s, fd);
        n5[j] = sed_update(q, q_up, s_up, h_up, h, fu, q, s, fd);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SED_KMAX; j++) {
        const int k = A.nivhau + (int)threadIdx.y + j * SED_LANES;
        if (!live || k > A.nivbas) continue;
        const size_t i = col + pl * (size_t)(k - 1);
        if (k <= A.nivh2o - 1) q3[i] = n3[j];
        q4[i] = n4[j];
        q5[i] = n5[j];
    }
}

// ---------------------------------------------------------------------------
// tropospheric forcing: tropo F:4498-4571, co_tropo F:4617-4636,
// ecmwfh2o F:8649-8655, fused (they write disjoint species of a cell)
// ---------------------------------------------------------------------------
// 1-based qj1 slots that tropo sets below nivbas (F:4502-4518), in the order of
// the forcing values
__constant__ int kTropoSlot[16] = {1, 2, 4, 7, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42};

struct ForcArgs {
    const double* pre;  // trajpre(:,:,:,irapp)
    double* qj1;
    double* hc;
    const double* co;   // co(nlon,nlat) of the month, or NULL: no co_tropo
    const double* hj1;  // hj1(nlon,nlat,niv), or NULL: no ecmwfh2o
    int nlon, nlat, niv, nivbas, nivh2o, kfirst, row0, nrows;
    int tropo;          // 1: tropo with v[]
    double v[16];
    double ox_decay;    // exp(-dtt/tau), tau 1 day (F:4528-4529)
    double co_decay;    // exp(-dtt/tau), tau 24 h (F:4612-4613)
};

__global__ void __launch_bounds__(128) k_forcing(ForcArgs A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nk = A.niv - A.kfirst + 1;
    if (t >= (long long)A.nlon * A.nrows * nk) return;
    const int ilon = (int)(t % A.nlon);
    const int r = (int)((t / A.nlon) % A.nrows);
    const int k = A.kfirst + (int)(t / ((long long)A.nlon * A.nrows));  // 1-based level
    const size_t pl = (size_t)A.nlon * A.nlat;
    const size_t i = (size_t)ilon + (size_t)A.nlon * (A.row0 + r) + pl * (size_t)(k - 1);
    const size_t p3 = pl * A.niv;
    double* q = A.qj1 + i;
    if (A.tropo && k >= A.nivbas + 1) {
#pragma unroll
        for (int n = 0; n < 16; n++) q[p3 * (kTropoSlot[n] - 1)] = A.v[n];
        const double q8 = q[p3 * 7];
        const double p = A.pre[i];
        const double ilim = p > 370. ? add(mul(-2.3825e-8, log(p)), 1.9457e-7) : q8;
        q[p3 * 7] = fmax(add(ilim, mul(sub(q8, ilim), A.ox_decay)), 0.);
    }
    if (A.tropo && k >= A.nivbas) {  // F:4548-4555: O3 and passive Ox = Ox
        const double q8 = q[p3 * 7];
        A.hc[i + p3 * 4] = q8;
        q[p3 * 10] = q8;
    }
    if (A.co && k >= A.nivbas + 1) {
        const double ilim = A.co[(size_t)ilon + (size_t)A.nlon * (A.row0 + r)];
        q[p3 * 8] = fmax(add(ilim, mul(sub(q[p3 * 8], ilim), A.co_decay)), 1.e-30);
    }
    if (A.hj1 && k >= A.nivh2o) q[p3 * 2] = dvd(mul(A.hj1[i], 28.97), 18.);
}

}  // namespace

// forcing values of tropo for a date (F:4414-4495): June values of the year
// before and after the date, interpolated linearly in time, then the lumped
// species (CFC-114/115 into CFC-12, HCFC-141b into CH3CCl3, HCFC-142b into
// HCFC-22, H-2402 into H-1301)
extern "C" int reprobus_tropo_values(int ian, int imois, double* v) {
    if (!v) return reprobus_set_error(REPROBUS_ERR_ARG, "v is NULL");
    if (imois < 1 || imois > 12) return reprobus_set_error(REPROBUS_ERR_ARG, "month %d outside 1..12", imois);
    const double yearccmval = (double)ian + (double)(imois - 1) / 12.;
    int icount = 0;
    double val[TROPO_NTAB];
    bool found = false;
    for (int iyear = TROPO_YEAR0; iyear < TROPO_YEAR0 + TROPO_NYEAR; iyear++) {
        icount++;
        if ((double)iyear + 0.5 > yearccmval) {
            // the reference then reads the table at icount - 1 = 0 (out of its
            // bounds) for dates before June 1988: refused here
            if (icount == 1) break;
            const double cinf = (yearccmval - (double)(iyear - 1) - 0.5) / 1.;
            const double csup = 1. - cinf;
            for (int n = 0; n < TROPO_NTAB; n++)
                val[n] = cinf * kTropoTab[n][icount - 1] + csup * kTropoTab[n][icount - 2];
            found = true;
            break;
        }
    }
    if (!found)
        return reprobus_set_error(REPROBUS_ERR_ARG,
                                  "date %d/%02d outside the forcing tables (June 1988 .. June 2024)", ian, imois);
    val[TT_CFC12] = val[TT_CFC12] + val[TT_CFC114] + 0.5 * val[TT_CFC115];
    val[TT_CH3CCL3] = val[TT_CH3CCL3] + val[TT_HCFC141B] * 2. / 3.;
    val[TT_HCFC22] = val[TT_HCFC22] + val[TT_HCFC142B];
    val[TT_H1301] = val[TT_H1301] + val[TT_H2402] * 2.;
    const int order[16] = {TT_N2O,   TT_CH4,   TT_NOY,  TT_CLY,   TT_CFC11, TT_CFC12,  TT_CFC113, TT_CCL4,
                           TT_CH3CCL3, TT_CH3CL, TT_HCFC22, TT_CH3BR, TT_H1211, TT_H1301, TT_BRY,    TT_CH2BR2};
    for (int n = 0; n < 16; n++) v[n] = val[order[n]];
    return REPROBUS_OK;
}

static int check_rows(const HandleInfo& H, int ilat0, int ilat1) {
    if (ilat0 < 1 || ilat1 > H.nlat || ilat0 > ilat1)
        return reprobus_set_error(REPROBUS_ERR_ARG, "rows %d..%d outside 1..%d", ilat0, ilat1, H.nlat);
    return REPROBUS_OK;
}

extern "C" int reprobus_sedimentation_dev(void* handle, int ilat0, int ilat1, const double* trajpre,
                                          const double* trajtem, int irapp, double* qj1, const double* vsed3d,
                                          int nivh2oecmwf, const double* parth2osed, const double* parthno3sed,
                                          double dtsedi) {
    HandleInfo H;
    int rc = handle_info(handle, &H);
    if (rc) return rc;
    if ((rc = check_rows(H, ilat0, ilat1))) return rc;
    if (irapp < 1 || irapp > H.nrappmax)
        return reprobus_set_error(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, H.nrappmax);
    if (!trajpre || !trajtem || !qj1 || !vsed3d || !parth2osed || !parthno3sed)
        return reprobus_set_error(REPROBUS_ERR_ARG, "NULL array argument");
    if (H.nivhau < 2) return reprobus_set_error(REPROBUS_ERR_ARG, "sedimentation needs nivhau >= 2 (got %d)", H.nivhau);
    if (H.nivbas - H.nivhau + 1 > SED_LANES * SED_KMAX)
        return reprobus_set_error(REPROBUS_ERR_ARG, "sedimentation covers at most %d levels (nivhau..nivbas)",
                                  SED_LANES * SED_KMAX);
    if (nivh2oecmwf < H.nivhau || nivh2oecmwf > H.nivbas + 1)
        return reprobus_set_error(REPROBUS_ERR_ARG, "nivh2oecmwf %d outside %d..%d", nivh2oecmwf, H.nivhau,
                                  H.nivbas + 1);
    SedArgs A;
    const size_t pl3 = (size_t)H.nlon * H.nlat * H.niv;
    A.pre = trajpre + (size_t)(irapp - 1) * pl3;
    A.tem = trajtem + (size_t)(irapp - 1) * pl3;
    A.qj1 = qj1;
    A.vsed = vsed3d;
    A.ph2o = parth2osed;
    A.pno3 = parthno3sed;
    A.nlon = H.nlon, A.nlat = H.nlat, A.niv = H.niv, A.nivbas = H.nivbas, A.nivhau = H.nivhau;
    A.nivh2o = nivh2oecmwf;
    A.row0 = ilat0 - 1;
    A.nrows = ilat1 - ilat0 + 1;
    A.dt = dtsedi;
    const int n = A.nlon * A.nrows;
    k_sediment<<<(n + SED_COLS - 1) / SED_COLS, dim3(SED_COLS, SED_LANES), 0, H.stream>>>(A);
    COL_TRY(cudaGetLastError());
    COL_TRY(cudaStreamSynchronize(H.stream));
    return REPROBUS_OK;
}

extern "C" int reprobus_forcing_dev(void* handle, int ilat0, int ilat1, int ian, int imois, double dt,
                                    const double* trajpre, int irapp, const double* co_month,
                                    const double* hj1, int nivh2oecmwf, double* qj1, double* hc) {
    HandleInfo H;
    int rc = handle_info(handle, &H);
    if (rc) return rc;
    if ((rc = check_rows(H, ilat0, ilat1))) return rc;
    if (irapp < 1 || irapp > H.nrappmax)
        return reprobus_set_error(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, H.nrappmax);
    if (!trajpre || !qj1 || !hc) return reprobus_set_error(REPROBUS_ERR_ARG, "NULL array argument");
    if (hj1 && (nivh2oecmwf < 1 || nivh2oecmwf > H.niv))
        return reprobus_set_error(REPROBUS_ERR_ARG, "nivh2oecmwf %d outside 1..%d", nivh2oecmwf, H.niv);
    ForcArgs A;
    memset(&A, 0, sizeof(A));
    if ((rc = reprobus_tropo_values(ian, imois, A.v))) return rc;
    A.tropo = 1;
    A.pre = trajpre + (size_t)(irapp - 1) * H.nlon * H.nlat * H.niv;
    A.qj1 = qj1;
    A.hc = hc;
    A.co = co_month;
    A.hj1 = hj1;
    A.nlon = H.nlon, A.nlat = H.nlat, A.niv = H.niv, A.nivbas = H.nivbas;
    A.nivh2o = hj1 ? nivh2oecmwf : H.niv + 1;
    A.kfirst = A.nivh2o < H.nivbas ? A.nivh2o : H.nivbas;
    A.row0 = ilat0 - 1;
    A.nrows = ilat1 - ilat0 + 1;
    // step constants, as the reference computes them once per call
    A.ox_decay = exp(-(dt / (24. * 60. * 60.)) / 1.);
    A.co_decay = exp(-(dt / (60. * 60.)) / 24.);
    const long long n = (long long)A.nlon * A.nrows * (A.niv - A.kfirst + 1);
    if (n > 0) {
        k_forcing<<<(unsigned)((n + 127) / 128), 128, 0, H.stream>>>(A);
        COL_TRY(cudaGetLastError());
    }
    COL_TRY(cudaStreamSynchronize(H.stream));
    return REPROBUS_OK;
}

// ---------------------------------------------------------------------------
// altitude, altitude.f90:1-148
// ---------------------------------------------------------------------------
namespace {

constexpr double kCtegas = 287.04 / 9.80665;  // R_dry / g at 45 degrees (altitude.f90:29)

struct GeoArgs {
    const double* relief;  // (nlon,nlat)
    const double* psol;    // (nlon,nlat)
    const double* aaa;     // (niv)
    const double* bbb;     // (niv)
    const double* t;       // (nlon,nlat,niv) regular grid
    const double* h2o;     // (nlon,nlat,niv) regular grid
    double* p;             // out: (nlon,nlat,niv) pressure of the regular grid
    double* tv;            // out: virtual temperature
    double* georeg;        // out: geopotential height (km)
    int* mono;             // out: (nlon,nlat) 1 when p increases with the level
    int nlon, nlat, niv;
};

// one thread per regular grid point: p and tv (altitude.f90:34-46) and the
// geopotential increment between the point and the one below it (:55-57; at
// the lowest level the step from the surface, :51-52), into georeg
__global__ void __launch_bounds__(128) k_geo_levels(GeoArgs A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t pl = (size_t)A.nlon * A.nlat;
    if (t >= (long long)pl * A.niv) return;
    const size_t c = (size_t)(t % pl);
    const int k = (int)(t / pl);  // 0-based level
    const double ps = A.psol[c];
    auto tv_at = [&](size_t i) { return mul(A.t[i], add(1., dvd(mul(mul(0.608, A.h2o[i]), 18.), 28.97))); };
    const double p = add(A.aaa[k], mul(A.bbb[k], ps));
    const double tv = tv_at(t);
    double inc;
    if (k == A.niv - 1) {
        inc = add(A.relief[c], mul(mul(mul(kCtegas, tv), log(dvd(ps, p))), 1.e-3));
    } else {
        const double p1 = add(A.aaa[k + 1], mul(A.bbb[k + 1], ps));
        inc = mul(mul(mul(kCtegas, dvd(add(tv_at(t + pl), tv), 2.)), log(dvd(p1, p))), 1.e-3);
    }
    A.p[t] = p;
    A.tv[t] = tv;
    A.georeg[t] = inc;
}

// one thread per regular column: the hypsometric sum from the surface up in
// the reference's order (:51-57), in place over the increments, and whether
// the pressure increases with the level
__global__ void __launch_bounds__(128) k_geo_sum(GeoArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nlon * A.nlat) return;
    const size_t pl = (size_t)A.nlon * A.nlat;
    double g = A.georeg[c + pl * (A.niv - 1)];
    double pk = A.p[c + pl * (A.niv - 1)];
    int mono = 1;
    for (int k = A.niv - 2; k >= 0; k--) {
        const size_t i = c + pl * k;
        g = add(g, A.georeg[i]);
        A.georeg[i] = g;
        const double p = A.p[i];
        if (!(p <= pk)) mono = 0;
        pk = p;
    }
    A.mono[c] = mono;
}

struct AltArgs {
    const double* trajlon;
    const double* trajlat;
    const double* trajpre;
    const double* p;
    const double* tv;
    const double* georeg;
    const int* mono;
    double* alt;
    int nlon, nlat, niv;
    double dlon, dlat;  // grid spacing (2 and 2 on the reference grid)
    double pi;
};

// one thread per trajectory point: nearest regular column (:61-74), the
// pressure clamp (:76-87: the reference's second statement overwrites the
// first, so only min(trajpre, p(niv)) acts), the highest regular level at or
// below it (:90-106: the smallest inivreg >= 2 with p >= pirr), the
// hypsometric step from there (:108-122) and the geometric altitude (:126-146)
__global__ void __launch_bounds__(128) k_altitude(AltArgs A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t pl = (size_t)A.nlon * A.nlat;
    if (t >= (long long)pl * A.niv) return;
    const double lon = A.trajlon[t], lat = A.trajlat[t];
    int il = (int)round(lon / A.dlon) + 1;
    if (il > A.nlon) il = 1;
    if (il < 1) il = 1;  // (not reached for longitudes in [0, 360))
    int jl = (int)round((90. - lat) / A.dlat) + 1;
    jl = jl < 1 ? 1 : (jl > A.nlat ? A.nlat : jl);  // (not reached for latitudes in [-90, 90])
    const size_t c = (size_t)(il - 1) + (size_t)A.nlon * (jl - 1);
    const double* p = A.p + c;  // p[pl * k], 0-based level k
    const double pirr = fmin(A.trajpre[t], p[pl * (A.niv - 1)]);
    int kr;  // 1-based
    if (A.mono[c]) {
        int lo = 2, hi = A.niv;  // p(hi) >= pirr always holds
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (p[pl * (mid - 1)] >= pirr)
                hi = mid;
            else
                lo = mid + 1;
        }
        kr = lo;
    } else {
        kr = A.niv;
        for (int k = 2; k <= A.niv; k++)
            if (p[pl * (k - 1)] >= pirr) {
                kr = k;
                break;
            }
    }
    const double* tv = A.tv + c;
    const double dz = mul(mul(dvd(mul(kCtegas, add(tv[pl * (kr - 1)], tv[pl * (kr - 2)])), 2.),
                              log(dvd(p[pl * (kr - 1)], pirr))),
                          1.e-3);
    const double geo = add(A.georeg[c + pl * (kr - 1)], dz);
    const double xlat = dvd(mul(lat, A.pi), 180.);
    const double c2 = cos(mul(2., xlat));
    A.alt[t] = add(mul(add(1., mul(0.002644, c2)), geo), dvd(mul(add(1., mul(0.0089, c2)), mul(geo, geo)), 6245.));
}

}  // namespace

extern "C" int reprobus_altitude_dev(void* handle, const double* relief, const double* psol, const double* aaa,
                                     const double* bbb, const double* t, const double* h2o, const double* trajlon,
                                     const double* trajlat, const double* trajpre, int irapp, double* alt) {
    HandleInfo H;
    int rc = handle_info(handle, &H);
    if (rc) return rc;
    if (irapp < 1 || irapp > H.nrappmax)
        return reprobus_set_error(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, H.nrappmax);
    if (!relief || !psol || !aaa || !bbb || !t || !h2o || !trajlon || !trajlat || !trajpre || !alt)
        return reprobus_set_error(REPROBUS_ERR_ARG, "NULL array argument");
    if (H.niv < 2 || H.nlat < 2) return reprobus_set_error(REPROBUS_ERR_ARG, "altitude needs niv >= 2 and nlat >= 2");
    const size_t pl = (size_t)H.nlon * H.nlat, n3 = pl * H.niv;
    void* scratch = nullptr;
    if ((rc = handle_scratch(handle, 3 * n3 * sizeof(double) + pl * sizeof(int), &scratch))) return rc;
    GeoArgs G;
    G.relief = relief, G.psol = psol, G.aaa = aaa, G.bbb = bbb, G.t = t, G.h2o = h2o;
    G.p = (double*)scratch;
    G.tv = G.p + n3;
    G.georeg = G.tv + n3;
    G.mono = (int*)(G.georeg + n3);
    G.nlon = H.nlon, G.nlat = H.nlat, G.niv = H.niv;
    k_geo_levels<<<(unsigned)((n3 + 127) / 128), 128, 0, H.stream>>>(G);
    k_geo_sum<<<(unsigned)((pl + 127) / 128), 128, 0, H.stream>>>(G);
    COL_TRY(cudaGetLastError());
    AltArgs A;
    const size_t off = (size_t)(irapp - 1) * n3;
    A.trajlon = trajlon + off, A.trajlat = trajlat + off, A.trajpre = trajpre + off;
    A.p = G.p, A.tv = G.tv, A.georeg = G.georeg, A.mono = G.mono;
    A.alt = alt;
    A.nlon = H.nlon, A.nlat = H.nlat, A.niv = H.niv;
    A.dlon = 360. / H.nlon;
    A.dlat = 180. / (H.nlat - 1);
    A.pi = 2. * asin(1.);
    k_altitude<<<(unsigned)((n3 + 127) / 128), 128, 0, H.stream>>>(A);
    COL_TRY(cudaGetLastError());
    COL_TRY(cudaStreamSynchronize(H.stream));
    return REPROBUS_OK;
}

// ---------------------------------------------------------------------------
// history / restart record, F:587-588 (write(78)) and F:231-235 (read(90))
//
// One Fortran sequential unformatted record, big-endian (the reference is
// built with -convert big_endian, reprobus-simulation.sh:133):
//   [4-byte length L] namexp(6 chars) ian imois ijour iheure imin (5 x int32)
//   pj1(nlon,nlat) uj1 vj1 alt tj1 (nlon,nlat,niv each) qj1(...,43)
//   surfarea(nlon,nlat,niv) hc(...,15) [4-byte length L]
// The FP64 arrays stay in HBM: k_swap64 reverses the byte order of a chunk of
// them straight into mapped pinned host memory (or back from it), so the host
// only moves bytes between the pinned buffers and the file. Records of 2^31
// bytes and more (subrecords) are refused.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ unsigned long long bswap64(unsigned long long v) {
    const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
    return ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
}

// n 8-byte words from src to dst with the byte order reversed; both 8-byte
// aligned (device or mapped pinned host memory)
__global__ void __launch_bounds__(256) k_swap64(unsigned long long* __restrict__ dst,
                                                const unsigned long long* __restrict__ src, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = bswap64(src[i]);
}

constexpr size_t kHistChunk = 8u << 20;  // 8-byte words per pinned buffer (64 MiB)

struct HistField {
    const double* src;  // write: device array
    double* dst;        // read: device array
    size_t n;           // words
};

void put_be32(unsigned char* b, unsigned v) {
    b[0] = (unsigned char)(v >> 24), b[1] = (unsigned char)(v >> 16), b[2] = (unsigned char)(v >> 8),
    b[3] = (unsigned char)v;
}
unsigned get_be32(const unsigned char* b) {
    return ((unsigned)b[0] << 24) | ((unsigned)b[1] << 16) | ((unsigned)b[2] << 8) | (unsigned)b[3];
}

struct Pinned {
    unsigned long long* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Pinned() {
        for (auto& b : buf)
            if (b) cudaFreeHost(b);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
    int init() {
        for (int i = 0; i < 2; i++) {
            COL_TRY(cudaHostAlloc((void**)&buf[i], kHistChunk * 8, cudaHostAllocMapped));
            COL_TRY(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        }
        return REPROBUS_OK;
    }
};

int swap_grid(size_t n) {
    const size_t b = (n + 255) / 256;
    return (int)(b < 4096 ? b : 4096);
}

size_t hist_fields(const HandleInfo& H, HistField* f, const double* const* src, double* const* dst) {
    const size_t pl = (size_t)H.nlon * H.nlat, p3 = pl * H.niv;
    const size_t n[8] = {pl, p3, p3, p3, p3, p3 * 43, p3, p3 * 15};
    size_t words = 0;
    for (int i = 0; i < 8; i++) {
        f[i].src = src ? src[i] : nullptr;
        f[i].dst = dst ? dst[i] : nullptr;
        f[i].n = n[i];
        words += n[i];
    }
    return words;
}

}  // namespace

extern "C" int reprobus_history_write_dev(void* handle, const char* path, const char* namexp, int ian, int imois,
                                          int ijour, int iheure, int imin, const double* pj1, const double* uj1,
                                          const double* vj1, const double* alt, const double* tj1, const double* qj1,
                                          const double* surfarea, const double* hc) {
    HandleInfo H;
    int rc = handle_info(handle, &H);
    if (rc) return rc;
    if (!path || !namexp || !pj1 || !uj1 || !vj1 || !alt || !tj1 || !qj1 || !surfarea || !hc)
        return reprobus_set_error(REPROBUS_ERR_ARG, "NULL argument");
    const double* src[8] = {pj1, uj1, vj1, alt, tj1, qj1, surfarea, hc};
    HistField f[8];
    const size_t words = hist_fields(H, f, src, nullptr);
    const size_t len = 6 + 5 * 4 + words * 8;
    if (len > 0x7fffffffULL)
        return reprobus_set_error(REPROBUS_ERR_ARG, "record of %zu bytes needs Fortran subrecords (not supported)", len);
    Pinned pin;
    if ((rc = pin.init())) return rc;
    FILE* fp = fopen(path, "wb");
    if (!fp) return reprobus_set_error(REPROBUS_ERR_ARG, "cannot open %s for writing", path);
    unsigned char head[4 + 6 + 20];
    put_be32(head, (unsigned)len);
    char name[6];
    memset(name, ' ', 6);  // character*6, blank padded
    for (int i = 0; i < 6 && namexp[i]; i++) name[i] = namexp[i];
    memcpy(head + 4, name, 6);
    const int date[5] = {ian, imois, ijour, iheure, imin};
    for (int i = 0; i < 5; i++) put_be32(head + 10 + 4 * i, (unsigned)date[i]);
    bool ok = fwrite(head, 1, sizeof(head), fp) == sizeof(head);
    // chunk c: swap into buffer c % 2 on the GPU, then write it; the swap of
    // chunk c+1 runs while chunk c is written
    int pend = -1;
    size_t pend_n = 0;
    int b = 0;
    for (int i = 0; i < 8 && ok; i++) {
        for (size_t o = 0; o < f[i].n && ok; o += kHistChunk) {
            const size_t n = f[i].n - o < kHistChunk ? f[i].n - o : kHistChunk;
            k_swap64<<<swap_grid(n), 256, 0, H.stream>>>(pin.buf[b], (const unsigned long long*)(f[i].src + o), n);
            cudaError_t e = cudaEventRecord(pin.ev[b], H.stream);
            if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                ok = false;
                break;
            }
            if (pend >= 0) {
                ok = cudaEventSynchronize(pin.ev[pend]) == cudaSuccess &&
                     fwrite(pin.buf[pend], 8, pend_n, fp) == pend_n;
            }
            pend = b, pend_n = n;
            b ^= 1;
        }
    }
    if (ok && pend >= 0)
        ok = cudaEventSynchronize(pin.ev[pend]) == cudaSuccess && fwrite(pin.buf[pend], 8, pend_n, fp) == pend_n;
    unsigned char tail[4];
    put_be32(tail, (unsigned)len);
    ok = ok && fwrite(tail, 1, 4, fp) == 4;
    ok = (fclose(fp) == 0) && ok;
    if (!ok) {
        cudaError_t e = cudaStreamSynchronize(H.stream);
        if (e != cudaSuccess) return reprobus_set_error(REPROBUS_ERR_CUDA, "history write: %s", cudaGetErrorString(e));
        return reprobus_set_error(REPROBUS_ERR_ARG, "history write to %s failed", path);
    }
    return REPROBUS_OK;
}

extern "C" int reprobus_history_read_dev(void* handle, const char* path, char* namexp, int* date, double* pj1,
                                         double* uj1, double* vj1, double* alt, double* tj1, double* qj1,
                                         double* surfarea, double* hc) {
    HandleInfo H;
    int rc = handle_info(handle, &H);
    if (rc) return rc;
    if (!path || !namexp || !date || !pj1 || !uj1 || !vj1 || !alt || !tj1 || !qj1 || !surfarea || !hc)
        return reprobus_set_error(REPROBUS_ERR_ARG, "NULL argument");
    double* dst[8] = {pj1, uj1, vj1, alt, tj1, qj1, surfarea, hc};
    HistField f[8];
    const size_t words = hist_fields(H, f, nullptr, dst);
    const size_t len = 6 + 5 * 4 + words * 8;
    FILE* fp = fopen(path, "rb");
    if (!fp) return reprobus_set_error(REPROBUS_ERR_ARG, "cannot open %s", path);
    unsigned char head[30];
    if (fread(head, 1, 30, fp) != 30) {
        fclose(fp);
        return reprobus_set_error(REPROBUS_ERR_ARG, "%s: short file", path);
    }
    if (get_be32(head) != len) {
        fclose(fp);
        return reprobus_set_error(REPROBUS_ERR_ARG, "%s: record of %u bytes, the grid %dx%dx%d needs %zu", path,
                                  get_be32(head), H.nlon, H.nlat, H.niv, len);
    }
    memcpy(namexp, head + 4, 6);
    namexp[6] = '\0';
    for (int i = 0; i < 5; i++) date[i] = (int)get_be32(head + 10 + 4 * i);
    Pinned pin;
    if ((rc = pin.init())) {
        fclose(fp);
        return rc;
    }
    // chunk c: read into buffer c % 2, then swap it into HBM on the GPU; the
    // read of chunk c+1 waits only for the swap of chunk c-1
    bool ok = true;
    int b = 0;
    bool used[2] = {false, false};
    for (int i = 0; i < 8 && ok; i++) {
        for (size_t o = 0; o < f[i].n && ok; o += kHistChunk) {
            const size_t n = f[i].n - o < kHistChunk ? f[i].n - o : kHistChunk;
            if (used[b] && cudaEventSynchronize(pin.ev[b]) != cudaSuccess) {
                ok = false;
                break;
            }
            if (fread(pin.buf[b], 8, n, fp) != n) {
                ok = false;
                break;
            }
            k_swap64<<<swap_grid(n), 256, 0, H.stream>>>((unsigned long long*)(f[i].dst + o), pin.buf[b], n);
            ok = cudaEventRecord(pin.ev[b], H.stream) == cudaSuccess && cudaGetLastError() == cudaSuccess;
            used[b] = true;
            b ^= 1;
        }
    }
    unsigned char tail[4];
    ok = ok && fread(tail, 1, 4, fp) == 4 && get_be32(tail) == len;
    fclose(fp);
    cudaError_t e = cudaStreamSynchronize(H.stream);
    if (e != cudaSuccess) return reprobus_set_error(REPROBUS_ERR_CUDA, "history read: %s", cudaGetErrorString(e));
    if (!ok) return reprobus_set_error(REPROBUS_ERR_ARG, "%s: truncated or malformed history record", path);
    return REPROBUS_OK;
}
