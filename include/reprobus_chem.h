/*
 * reprobus_chem.h — C-ABI of the GB300 (sm_103a) REPROBUS chemistry step.
 *
 * The library libreprobus_gb300.so replaces the per-latitude chemistry loop of
 * the REPROBUS time loop:
 *
 *     do ilat = 1,nlat
 *        call chem3d(ilat, daynum, dt, alt, trajlon, trajlat, trajpre,
 *                    trajtem, irapp, qj1, hc, vsed3d, parth2osed,
 *                    parthno3sed, surfarea, sza3d)
 *     end do                          ! src/reprobus_l137_20230723.f:398-415
 *     call conserv(qj1, hc)           ! :427   (optional, REPROBUS_FUSE_CONSERV)
 *     qj1(:,:,:,1:42) >= 1e-30        ! :431-440
 *     qj1(:,:,nivbas+1:,43) = qj1(..,5) ! :444-450
 *
 * Conventions (all entry points):
 *  - Arrays are FP64 in Fortran (column-major) layout, lon fastest, exactly
 *    as the reference declares them: qj1(nlon,nlat,niv,43), hc(nlon,nlat,niv,15),
 *    alt/surfarea(nlon,nlat,niv), traj*(nlon,nlat,niv,nrappmax),
 *    vsed3d/parth2osed/parthno3sed/sza3d(nlon,nlat,nivbas).
 *  - Indices that the Fortran caller passes (ilat, irapp) are 1-based.
 *  - Plain pointers and sizes only; the caller owns every array.
 *  - Return 0 on success, a REPROBUS_ERR_* code otherwise; the text of the
 *    last error of the calling thread is in reprobus_last_error().
 *  - A handle owns its device buffers and one CUDA stream. It is not
 *    thread-safe: one host thread drives a handle at a time.
 *  - No entry point falls back to the CPU: without a usable GPU the calls
 *    return REPROBUS_ERR_NODEVICE / REPROBUS_ERR_CUDA.
 */
#ifndef REPROBUS_CHEM_H
#define REPROBUS_CHEM_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
    REPROBUS_OK = 0,
    REPROBUS_ERR_ARG = 1,        /* null pointer, bad size, bad row/slice index   */
    REPROBUS_ERR_CUDA = 2,       /* a CUDA runtime call failed                    */
    REPROBUS_ERR_NONFINITE = 3,  /* NaN/Inf written by the step (see stats)       */
    REPROBUS_ERR_NOCONV = 4,     /* solver: cells left unconverged (see stats)    */
    REPROBUS_ERR_TIMEOUT = 5,    /* a bounded device-side wait gave up            */
    REPROBUS_ERR_NODEVICE = 6    /* no CUDA device visible                        */
};

/* ---- handle flags --------------------------------------------------------- */
#define REPROBUS_FUSE_CONSERV  0x1  /* also run conserv (:2526-2616), clamps and
                                       the HNO3-gas copy (:431-450) in the call  */
#define REPROBUS_CHECK_FINITE  0x2  /* count NaN/Inf in outputs, return
                                       REPROBUS_ERR_NONFINITE when any           */
#define REPROBUS_USE_GRAPH     0x4  /* launch the step as one CUDA graph (each
                                       solver configuration runs once directly
                                       first; the graph is captured per call and
                                       updated in place)                         */

/* ---- solvers (reprobus_chem_set_solver) ----------------------------------- */
#define REPROBUS_SOLVER_REF5          0  /* the reference scheme: niter fixed passes  */
#define REPROBUS_SOLVER_NEWTON64      1  /* Newton to the fixed point, FP64 Jacobian   */
#define REPROBUS_SOLVER_NEWTON_MIXED  2  /* Newton, FP32 Jacobian and LU, FP64 residual
                                            and update                                 */

/* ---- per-call statistics --------------------------------------------------- */
typedef struct reprobus_stats {
    long long ncells;          /* cells integrated by the call (rows x nlon x nivbas) */
    long long nonfinite;       /* NaN/Inf values produced (REPROBUS_CHECK_FINITE)     */
    int kernel_launches;       /* kernels this call launched                          */
    int passes;                /* reference passes per cell (niter, or Newton's npass) */
    double device_ms;          /* device time of the call's kernels (CUDA events)      */
    long long newton_iters;    /* Newton solvers: iterations summed over converged cells */
    long long fallbacks;       /* Newton solvers: cells that fell back to the passes  */
    int max_newton_iters;      /* Newton solvers: most iterations one cell needed     */
    int solver;                /* REPROBUS_SOLVER_* used                              */
    int lanes_per_block;       /* Newton solvers: cells in flight per block of the
                                  persistent solve kernel (autotuned or set)         */
    int blocks_per_sm;         /* Newton solvers: resident blocks of it per SM        */
    int z_shared;              /* Newton solvers: 1 when the kernel keeps the right-
                                  hand side in shared memory, 0 in registers, 2 in
                                  registers with two warp groups sharing the matrix
                                  slots, 3 with a residual lane per cell, 4 in
                                  registers with the block's warps in lock-step  */
    int warm_start;            /* Newton solvers: 1 when a network for the learned
                                  restart is attached                                */
    long long warm_restarts;   /* learned restart: cells whose plain start missed the
                                  convergence test and that were solved again from
                                  the network's prediction                           */
    long long failed_iters;    /* Newton solvers: iterations of attempts that did not
                                  converge (plain starts that missed, fallbacks)     */
    double solve_ms;           /* Newton solvers: device time of the persistent solve
                                  kernel (its first launch)                          */
    int graph;                 /* 1 when the step ran as a CUDA graph               */
    long long start64_cells;   /* mixed solver: cells whose FP32 start passes left
                                  the FP32 range and were started in FP64        */
} reprobus_stats;

/* ---- diagnostics layout (reprobus_chem_rates_*) ----------------------------
 * Per chemistry cell, REPROBUS_DIAG_COUNT doubles, stored structure-of-arrays:
 * diag[d * ncell + cell], cell = ilon-1 + nlon*((ilat-ilat0) + nrows*(iniv-1)).
 * The 99 rate constants follow the order of src/reprobus_l137_20230723.f:930-1303
 * (a1 a1et a2 a5 a6 a6b a7 a17 a19 a26 a27 a30 a31 a36 | b3 b4 b6 b7 b9 b12 b22
 *  b23 b24 b27 b28 b32 b38 b39 | c1a c1b c1c c2 c3 c4 c5 c7 c8 c9 c10 c12 c14
 *  c15 c17a c17b c18 c19 | d2 d3 d4 d5 d6 d7 d8 d9 d10 d11 d31 d32 d33 d34 d35
 *  d36 d37 d60 d61 d62 d90 d91 d92 d93 d94 d95 d96 d97 | e2 e3 e4 e5a e5b e5c e6
 *  e7 e8 e9 e10 e11 e13 e15 e16 e50 e51 e52 e53 e54 | hk1 hk2 hk3 hk4 hk5). */
enum {
    REPROBUS_DIAG_HNM = 0,
    REPROBUS_DIAG_SZA = 1,
    REPROBUS_DIAG_O3T = 2,
    REPROBUS_DIAG_TJ = 3,            /* 41 photolysis rates, :754-794 order     */
    REPROBUS_DIAG_HET = 44,          /* het1..het9                              */
    REPROBUS_DIAG_PARTHNO3 = 53,
    REPROBUS_DIAG_PARTHNO3SL = 54,
    REPROBUS_DIAG_PARTH2O = 55,
    REPROBUS_DIAG_PARTHCL = 56,
    REPROBUS_DIAG_VSED = 57,
    REPROBUS_DIAG_SURFAREA = 58,     /* levels nivhau..nivbas, else 0            */
    REPROBUS_DIAG_RATE = 59,         /* 99 thermal rate constants               */
    REPROBUS_DIAG_COUNT = 158
};
#define REPROBUS_NRATE 99
#define REPROBUS_NBCON 43           /* transported slots qj1(...,43)            */
#define REPROBUS_NCM 15             /* steady-state slots hc(...,15)            */
#define REPROBUS_NPHOT 41
#define REPROBUS_NZ 101
#define REPROBUS_NSZA 27
#define REPROBUS_NOZO 7
#define REPROBUS_NTROE 18

/* Library version string. */
const char* reprobus_version(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char* reprobus_last_error(void);

/* Fills troe[18] with the fall-off prefactors of COMMON /constant/ in COMMON
 * order (a0hox a1hox a0nox1 a1nox1 a0nox2 a1nox2 a0nox3 a1nox3 a0clx1 a1clx1
 * a0clx2 a1clx2 a0clx3 a1clx3 a0brx a1brx a0c1 a1c1).
 * Replaces: subroutine const, src/reprobus_l137_20230723.f:5927-5948.
 * Host-only arithmetic; needs no GPU. */
int reprobus_chem_troe(double* troe);

/* Creates a handle: uploads the photolysis table ajl(40,101,27,7) (Fortran
 * order) and o3up(0:79) of COMMON /photodis/, and the 18 Troe prefactors of
 * COMMON /constant/; sizes the device buffers for the grid.
 * Replaces: call const(relief), :294, i.e. the COMMON blocks filled at
 * :5927-5973 and declared at :46-52.
 * nivbas: last chemistry level (reference: 94); nivhau: first PSC/aerosol
 * level (reference: 14); niter: fixed-point passes (reference: 5, :630).
 * Troe prefactors that are not positive and finite are refused with
 * REPROBUS_ERR_ARG (the rate stage works with their logarithms). */
int reprobus_chem_init(const double* ajl, const double* o3up, const double* troe,
                       int nlon, int nlat, int niv, int nivbas, int nivhau,
                       int nrappmax, int niter, int flags, void** handle);

/* Releases the handle and its device memory. */
int reprobus_chem_free(void* handle);

/* Makes the handle launch on the caller's CUDA stream (a cudaStream_t passed
 * as void*; NULL restores the handle's own stream). */
int reprobus_chem_set_stream(void* handle, void* cuda_stream);

/* Switches REPROBUS_USE_GRAPH on or off for the handle. No counterpart in
 * the reference. */
int reprobus_chem_set_graph(void* handle, int on);

/* Selects how the cells are integrated (default REPROBUS_SOLVER_REF5).
 * The Newton solvers return the fixed point of the reference's pass map
 * (:1350-2372) -- the step the reference's iteration approximates with its
 * 5 passes: npass reference passes from the start state, then Newton on the
 * equations generated from the pass (reprobus_gb300/codegen/gen_newton.py)
 * until the largest step relative to max(|x|, 1e-20 hnm) is below tol, at
 * most maxit iterations; a cell that does not converge falls back to the
 * reference's niter passes and is counted in stats.fallbacks.
 * Defaults: npass 5, maxit 12, tol 1e-4 (Newton converges superlinearly: the
 * step that passes the test is followed by none, and the answer lies within
 * ~1e-8 of the fixed point, far inside the 1e-6 accuracy target; 5 passes are
 * the fastest start of both solvers on the 2 x 2 degree grid). The network
 * of the learned restart (reprobus_chem_set_mlp) is trained for one npass
 * and must be used with it. No counterpart in the reference. */
int reprobus_chem_set_solver(void* handle, int solver, int npass, int maxit, double tol);

/* Shape of the persistent Newton solve kernel. lanes_per_block = 0 (default):
 * the first Newton step of each matrix precision times every compiled shape
 * (lanes per block x right-hand side in registers or shared memory x
 * resident blocks per SM) on that step's own cells and keeps the fastest
 * (synchronous, once per handle); > 0: use that many lanes per block (a
 * compiled value: 64, 96, 128 (zshared 0, 1) or 128, 256 (zshared 2) for the
 * mixed solver; 32, 64 (zshared 0, 1) or 64, 128 (zshared 2) for the FP64
 * one; a precision without that value is autotuned), zshared (0: right-hand
 * side in registers, 1: in shared memory, 2: in registers with two warp
 * groups taking turns on one set of matrix slots, so that a block keeps
 * twice the cells in flight; 3: in shared memory, with a second lane per cell
 * that evaluates the FP64 residual while the first evaluates the Jacobian;
 * lanes_per_block then counts cells: 64, 128 mixed, 32, 64 FP64; 4: in
 * registers, the warps of a block passing each phase of an iteration
 * together, so that they fetch the same code: 64, 128 mixed, 32, 64 FP64;
 * 5, 6: in shared memory, 2 or 4 warps per cell: the warps working on the
 * same 32 cells share out the rows of the Jacobian and of the residual, one
 * of them factorises and updates; lanes_per_block then counts cells: 32, 64
 * (5) and 32 (6) mixed, 32 FP64) and blocks_per_sm (0: as many as fit).
 * When the environment variable REPROBUS_TUNE_CACHE names a file, the
 * autotuner first looks there for a choice made for the same GPU model,
 * matrix precision and cell count (skipping the timing runs), and appends
 * each new choice to it. No counterpart in the reference. */
int reprobus_chem_set_tuning(void* handle, int lanes_per_block, int blocks_per_sm, int zshared);

/* ---- learned restart -------------------------------------------------------
 * A 64-256-256-256-64 MLP (SiLU; BF16 weights and activations, FP32
 * accumulation on the tensor cores) maps the 64 features of a cell at the
 * Newton solvers' plain start (npass reference passes from the start state):
 * log10 of its 42 transported and 15 short-lived mixing ratios floored at
 * 1e-30, T [K], ln p [hPa], cos(sza), log10 of the aerosol surface area
 * floored at 1e-12, latitude [deg], time of day [fraction], 0; to the log10
 * ratios of the 57 end-of-step mixing ratios to those of the plain start.
 * None of this has a counterpart in the reference. Device pointers
 * throughout; B rows of 64 FP32 values, row-major. */
#define REPROBUS_MLP_FEATURES 64
#define REPROBUS_MLP_OUTPUTS 64   /* 57 used */
#define REPROBUS_MLP_NNORM 320    /* in_mean[64] in_std[64] out_mean[64] out_std[64] out_min[64]:
                                     predictions with |y| < out_min are replaced by 0 */

/* Creates a network with He-uniform weights from seed and a training batch
 * capacity (a multiple of 128). */
int reprobus_mlp_create(int batch_cap, unsigned long long seed, void** net);
int reprobus_mlp_free(void* net);
/* Number of FP32 parameters, packed W0 b0 W1 b1 W2 b2 W3 b3 (W row-major,
 * fan_out x fan_in). */
int reprobus_mlp_nparams(void);
/* Host copies of the parameters and of the normalisation (either may be NULL). */
int reprobus_mlp_set_params(void* net, const float* params, const float* norm);
int reprobus_mlp_get_params(void* net, float* params, float* norm);
/* One Adam step (lr) on a batch (B a multiple of 128 up to batch_cap) of raw
 * features X and raw targets Y; *loss (nullable, host): mean squared error of
 * the normalised outputs before the step. */
int reprobus_mlp_train_step(void* net, const float* X, const float* Y, int B, float lr, float* loss,
                            void* cuda_stream);
/* Gradients of that loss (host, packed like the parameters) without a step. */
int reprobus_mlp_grads(void* net, const float* X, const float* Y, int B, float* grads, float* loss,
                       void* cuda_stream);
/* Inference on B rows (any B): Y = network(X), raw units. */
int reprobus_mlp_forward(void* net, const float* X, float* Y, int B, void* cuda_stream);
/* Fault handling hook: the number of polls after which the inference
 * kernel's waits on its weight copies and tensor-core work give up (polls < 0:
 * the default, 2^24; 0: the first wait gives up at once). A wait that gives
 * up makes the kernel skip its remaining work, wait (with the default limit)
 * for the copies and MMAs it has in flight, release its tensor memory and
 * report REPROBUS_ERR_TIMEOUT; the network stays usable. No counterpart in
 * the reference. */
int reprobus_mlp_set_wait_limit(void* net, long long polls);

/* Attaches a network to a chemistry handle (NULL detaches). The Newton
 * solvers then give a cell whose plain start misses the convergence test a
 * second attempt from the network's prediction for that plain start
 * (stats.warm_restarts; at most 65,536 cells per step), and only a cell that
 * misses again falls back to the reference passes. Every other cell's answer
 * is the same with and without the network. If the inference kernel gives up
 * waiting, those cells are solved again from the plain start (the answer
 * stands) and a call that reads the step's counters (stats requested, or
 * REPROBUS_CHECK_FINITE) returns REPROBUS_ERR_TIMEOUT. */
int reprobus_chem_set_mlp(void* handle, void* net);

/* The 64 raw features of every chemistry cell of rows ilat0..ilat1 at the
 * plain start of a step of length dt (the handle's npass reference passes;
 * device arrays as for reprobus_chem_rates_dev; feat: ncell x 64 FP32,
 * 16-byte aligned, cells in the diagnostics order). */
int reprobus_chem_features_dev(void* handle, int ilat0, int ilat1, double daynum, double dt, const double* alt,
                               const double* trajlon, const double* trajlat, const double* trajpre,
                               const double* trajtem, int irapp, const double* qj1, const double* hc,
                               float* feat);

/* One 15-min chemistry step for latitude rows ilat0..ilat1 (1-based,
 * inclusive), HOST arrays: copies the rows in, integrates, copies them back.
 * Replaces: do ilat = ilat0,ilat1 / call chem3d(...) (:398-415, chem3d at
 * :601-2412); with REPROBUS_FUSE_CONSERV also conserv (:427, :2526-2616) and
 * the clamps (:431-450) on those rows. Writes qj1/hc (levels 1..nivbas; with
 * the flag also the clamps on all levels), vsed3d, parth2osed, parthno3sed,
 * sza3d (levels 1..nivbas) and surfarea (levels nivhau..nivbas).
 * With 32 rows or more the rows go in 4 chunks, the copies of one chunk
 * overlapping the integration of the next; the environment variable
 * REPROBUS_HOST_CHUNKS (1..4) sets another number of chunks. */
int reprobus_chem_step(void* handle, int ilat0, int ilat1, double daynum, double dt,
                       const double* alt, const double* trajlon, const double* trajlat,
                       const double* trajpre, const double* trajtem, int irapp,
                       double* qj1, double* hc, double* vsed3d, double* parth2osed,
                       double* parthno3sed, double* surfarea, double* sza3d,
                       reprobus_stats* stats);

/* Same step on DEVICE arrays (full-grid Fortran layout, already resident in
 * HBM): no host<->device copies. Same replacement as reprobus_chem_step. */
int reprobus_chem_step_dev(void* handle, int ilat0, int ilat1, double daynum, double dt,
                           const double* alt, const double* trajlon, const double* trajlat,
                           const double* trajpre, const double* trajtem, int irapp,
                           double* qj1, double* hc, double* vsed3d, double* parth2osed,
                           double* parthno3sed, double* surfarea, double* sza3d,
                           reprobus_stats* stats);

/* Rate stage only (setup :800-833, total, zenith, phot+jno, analytic+hetero,
 * rate constants :920-1306) on DEVICE arrays; writes the per-cell
 * diagnostics (REPROBUS_DIAG_* layout) to diag. Does not modify the state.
 * Replaces: the part of chem3d before its iteration loop (:800-1338). */
int reprobus_chem_rates_dev(void* handle, int ilat0, int ilat1, double daynum,
                            const double* alt, const double* trajlon, const double* trajlat,
                            const double* trajpre, const double* trajtem, int irapp,
                            const double* qj1, const double* hc, double* diag);

/* Element conservation + clamps on DEVICE arrays, rows ilat0..ilat1.
 * Replaces: call conserv(qj1, hc) (:427, :2526-2616) and the loops at
 * :431-450. */
int reprobus_conserv_dev(void* handle, int ilat0, int ilat1, double* qj1, double* hc);

/* ---- column physics around the chemistry step ------------------------------
 * The other per-column work of the chemistry sub-step of the time loop
 * (:370-450), on DEVICE arrays in the reference's layout. Each call
 * synchronises the handle's stream before it returns. */

/* Sedimentation of H2O (levels nivhau..nivh2oecmwf-1), NOy and HNO3 (levels
 * nivhau..nivbas) for rows ilat0..ilat1, from the settling velocities and
 * non-sedimenting fractions that the chemistry step wrote (vsed3d,
 * parth2osed, parthno3sed), over the time step dtsedi. Needs nivhau >= 2,
 * nivhau <= nivh2oecmwf <= nivbas + 1 and at most 128 levels nivhau..nivbas.
 * Replaces: call sedimentation(trajpre, trajtem, irapp, qj1, vsed3d,
 * nivh2oecmwf, parth2osed, parthno3sed, dtsedi) (:420-422, routine
 * :2416-2522), which the reference runs after the last chemistry sub-step of
 * a transport step and before conserv. */
int reprobus_sedimentation_dev(void* handle, int ilat0, int ilat1, const double* trajpre,
                               const double* trajtem, int irapp, double* qj1, const double* vsed3d,
                               int nivh2oecmwf, const double* parth2osed, const double* parthno3sed,
                               double dtsedi);

/* The 16 tropospheric forcing mixing ratios of tropo for year ian, month imois
 * (June values of the years around the date, linear in time, lumped species
 * added), in the order of the qj1 slots 1 2 4 7 31..42 they set. Dates before
 * June 1988 or from June 2024 on are refused (the reference's tables end
 * there). Host only. Replaces: the date interpolation of tropo (:4414-4495). */
int reprobus_tropo_values(int ian, int imois, double* v);

/* Tropospheric forcing of rows ilat0..ilat1 for the date (ian, imois) and
 * step dt: tropo (levels nivbas+1..niv set to the forcing values, Ox relaxed
 * with a 1-day time constant, O3 and passive Ox = Ox from level nivbas);
 * co_tropo when co_month (nlon,nlat: the MOPITT CO field of the month) is
 * non-NULL; ecmwfh2o (H2O = hj1 x 28.97/18 from level nivh2oecmwf) when hj1
 * (nlon,nlat,niv: the ECMWF specific humidity at the step's time) is non-NULL.
 * Replaces: call tropo(ian, imois, dt, trajpre, irapp, qj1, hc) (:373,
 * routine :4077-4574), call co_tropo(imois, dt, qj1) (:377, :4577-4639) and
 * call ecmwfh2o(daynum, qj1, nivh2oecmwf, ...) (:382, :8621-8658); the
 * reference reads the CO and humidity fields from files (mopitt_corrected.txt,
 * ECMWF analyses): here the caller passes them. */
int reprobus_forcing_dev(void* handle, int ilat0, int ilat1, int ian, int imois, double dt,
                         const double* trajpre, int irapp, const double* co_month, const double* hj1,
                         int nivh2oecmwf, double* qj1, double* hc);

/* Geometric altitude (km) of every trajectory point (slice irapp of traj*)
 * from the regular grid's surface pressure psol(nlon,nlat), relief
 * (nlon,nlat), hybrid coefficients aaa(niv) [hPa] and bbb(niv), temperature
 * t(nlon,nlat,niv) and H2O mixing ratio h2o(nlon,nlat,niv); writes
 * alt(nlon,nlat,niv). The nearest regular column of a point uses the grid
 * spacing 360/nlon x 180/(nlat-1) (2 x 2 degrees on the reference grid, where
 * the reference hard-codes 2). Uses device scratch of the handle (3 doubles
 * per grid point).
 * Replaces: call altitude(nlon, nlat, niv, relief, pj1, aaa, bbb, tj1,
 * qj1(:,:,:,3), trajlon(:,:,:,irapp), trajlat(..), trajpre(..), alt) (:391-394,
 * routine altitude.f90:1-148). */
int reprobus_altitude_dev(void* handle, const double* relief, const double* psol, const double* aaa,
                          const double* bbb, const double* t, const double* h2o, const double* trajlon,
                          const double* trajlat, const double* trajpre, int irapp, double* alt);

/* History / restart record of the model state in the reference's file
 * format: one big-endian Fortran sequential unformatted record (4-byte length
 * markers) holding namexp (6 characters, blank padded), ian, imois, ijour,
 * iheure, imin (int32), pj1(nlon,nlat), uj1, vj1, alt, tj1 (nlon,nlat,niv),
 * qj1(...,43), surfarea(nlon,nlat,niv), hc(...,15). Arrays are DEVICE arrays;
 * the byte order is reversed on the GPU through mapped pinned buffers.
 * Records of 2^31 bytes or more are refused.
 * Replaces: write(78) namexp, ian, ..., hc (:587-588). */
int reprobus_history_write_dev(void* handle, const char* path, const char* namexp, int ian, int imois,
                               int ijour, int iheure, int imin, const double* pj1, const double* uj1,
                               const double* vj1, const double* alt, const double* tj1, const double* qj1,
                               const double* surfarea, const double* hc);

/* Reads such a record into DEVICE arrays; namexp gets 7 bytes (6 characters
 * and a NUL), date the 5 integers. A record whose length does not match the
 * handle's grid is refused. Replaces: read(90) namexp, ian, ..., hc
 * (:231-235). */
int reprobus_history_read_dev(void* handle, const char* path, char* namexp, int* date, double* pj1,
                              double* uj1, double* vj1, double* alt, double* tj1, double* qj1,
                              double* surfarea, double* hc);

/* Allocation-free variant of reprobus_chem_step_dev. No counterpart in the
 * reference: REPROBUS allocates all of its arrays itself, on the host.
 *
 * For callers that may not allocate device memory while they run: models
 * whose GPU memory is reserved once and handed out by their own runtime or
 * pool (OpenACC/CUDA-Fortran data regions, a framework's caching allocator),
 * or processes held to a fixed device-memory budget. The call needs no handle
 * and calls no cudaMalloc/cudaFree: the caller passes every array as a DEVICE
 * pointer -- the photolysis table ajl(40,101,27,7) and o3up(0:79) included --
 * plus the 18 Troe prefactors as a HOST array, and the step's only scratch
 * (3 doubles per chemistry cell + 1 per column + a counter) lives in one
 * fixed device array of REPROBUS_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB),
 * which every GPU that loads the library holds until the process exits.
 * Limit: 3*nlon*nrows*nivbas + nlon*nrows + 32 <= REPROBUS_NOALLOC_SCRATCH_DOUBLES
 * (reference grid, nivbas 94: up to 20 latitude rows per call); larger
 * requests return REPROBUS_ERR_ARG and do nothing.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before capturing
 * any stream. All calls share the one array and it keeps the last call's
 * contents: calls whose kernels overlap on the GPU (other streams, other host
 * threads) race on it; serialise them. A process that resets the device
 * (cudaDeviceReset) gets the address looked up again at its next call.
 * The call always integrates with the reference scheme (niter fixed passes,
 * REPROBUS_SOLVER_REF5): it has no handle, so no solver selection, Newton
 * state or network. Launches on `stream` (NULL: the default stream);
 * asynchronous unless REPROBUS_CHECK_FINITE is set, in which case it
 * synchronises to read the non-finite count. It runs the kernels of
 * reprobus_chem_step_dev with the same flags. Troe prefactors that are not
 * positive and finite are refused with REPROBUS_ERR_ARG. */
#define REPROBUS_NOALLOC_SCRATCH_DOUBLES (1 << 20)
int reprobus_chem_step_noalloc(const double* ajl, const double* o3up, const double* troe,
                               int nlon, int nlat, int niv, int nivbas, int nivhau,
                               int nrappmax, int niter, int flags, int ilat0, int ilat1,
                               double daynum, double dt, const double* alt,
                               const double* trajlon, const double* trajlat,
                               const double* trajpre, const double* trajtem, int irapp,
                               double* qj1, double* hc, double* vsed3d, double* parth2osed,
                               double* parthno3sed, double* surfarea, double* sza3d,
                               void* stream);

#ifdef __cplusplus
}
#endif
#endif /* REPROBUS_CHEM_H */
