/*
 * chem_oracle.h — CPU FP64 oracle of the REPROBUS chemistry step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker for the CUDA path: the tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it; the
 * product library never links or calls it.
 *
 * PARITY UNPINNED: the reference ships no tests, golden vectors or fixtures,
 * and it is Fortran 77 with no Fortran compiler in this image, so neither the
 * reference itself nor any output of it can be run here. The oracle restates
 * the reference routines statement by statement (file:line cited at each
 * function) and is pinned only by known-answer tests derived from the code.
 *
 * Array conventions follow the reference (Fortran column-major, FP64, lon
 * fastest); row/slice indices passed here are 0-based.
 */
#ifndef REPROBUS_CHEM_ORACLE_H
#define REPROBUS_CHEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_grid {
    int nlon, nlat, niv;   /* array extents (reference: 180, 91, 137)            */
    int nivbas;            /* last chemistry level, 1-based (reference: 94)      */
    int nivhau;            /* first aerosol level, 1-based (reference: 14)       */
    int nrappmax;          /* trajectory slices (reference: 12)                  */
    int niter;             /* fixed passes (reference: 5); <=0: iterate to tol   */
    double tol;            /* niter<=0: stop when max rel. change < tol          */
    int maxiter;           /* niter<=0: cap on passes                            */
    const double* ajl;     /* ajl(40,101,27,7)                                   */
    const double* o3up;    /* o3up(0:79)                                         */
    double troe[18];       /* COMMON /constant/                                  */
    int newton;            /* 1: after niter passes, Newton on the pass map to tol */
    int* cellstat;         /* nullable, per chemistry cell (diag layout): Newton
                              steps over all stages, >= 0 when converged,
                              -steps-1 when not                                   */
    double* cellres;       /* nullable, per chemistry cell: final max|G(x)-x|/scale */
    const double* x_qj1;   /* nullable: evaluate one pass G at the state x =    */
    const double* x_hc;    /* (x_qj1, x_hc) (mixing ratios, full arrays) instead
                              of iterating; cellres gets max|G(x)-x|/scale and
                              qj1/hc get G(x). With newton set: Newton (stage 1
                              alone) from x instead of from the 5-pass state     */
    int* cellstage;        /* nullable, per chemistry cell: the Newton stage that
                              converged (1: from the 5-pass state, 2-5: from the
                              0/1/2/3-pass state, 6: continuation; 0: none)       */
} orc_grid;

/* const, :5927-5948 — fills the 18 Troe prefactors. */
void orc_const(double* troe);

/* chem3d for latitude row ilat (0-based), :601-2412.
 * diag (nullable): per chemistry cell REPROBUS_DIAG_COUNT values, SoA over the
 * full grid's chemistry cells: diag[d*ncd + i + nlon*(ilat + nlat*k)],
 * ncd = nlon*nlat*nivbas.  passes (nullable): passes made in this row. */
void orc_chem3d(const orc_grid* g, int ilat, double daynum, double dt,
                const double* alt, const double* trajlon, const double* trajlat,
                const double* trajpre, const double* trajtem, int irapp,
                double* qj1, double* hc, double* vsed3d, double* parth2osed,
                double* parthno3sed, double* surfarea, double* sza3d,
                double* diag, int* passes);

/* conserv, :2526-2616, rows ilat0..ilat1 (0-based, inclusive). */
void orc_conserv(const orc_grid* g, int ilat0, int ilat1, double* qj1, double* hc);

/* clamps and HNO3-gas copy, :431-450, rows ilat0..ilat1. */
void orc_clamp(const orc_grid* g, int ilat0, int ilat1, double* qj1);

/* The time-loop chemistry block for rows ilat0..ilat1: chem3d per row
 * (:398-415), then (if fuse) conserv (:427) and clamps (:431-450).
 * nthreads: OpenMP threads over rows (<=0: all).  Returns max passes. */
int orc_step(const orc_grid* g, int ilat0, int ilat1, double daynum, double dt,
             const double* alt, const double* trajlon, const double* trajlat,
             const double* trajpre, const double* trajtem, int irapp,
             double* qj1, double* hc, double* vsed3d, double* parth2osed,
             double* parthno3sed, double* surfarea, double* sza3d,
             int fuse, double* diag, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
