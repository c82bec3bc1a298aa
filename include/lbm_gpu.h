/*
 * lbm_gpu.h - C ABI of the GB300 (sm_103a) coupled thermal MRT lattice-Boltzmann library.
 *
 * The reference (Fortran, 2DRB/2DRB.F90 and 2DRB/3DRB.F90) keeps its state in module
 * globals and advances it with argument-less subroutines called in a fixed order from
 * `program main` (2DRB.F90:236-277, 3DRB.F90:225-264).  This header replaces that
 * surface one to one: a handle owns the lattice (all of it resident in HBM on one
 * GPU), every reference subroutine on the time-step path has an entry point of the
 * same name, and `lbm_step` runs the fused GB300 kernels for many steps at once.
 *
 * Conventions
 *  - Every call returns an `int` status (LBM_OK = 0).  The library never exits the
 *    process; `lbm_last_error` gives the message of the last failure on a handle.
 *  - Calls enqueue work on the handle's own CUDA stream.  Only calls that return
 *    host data (getters and diagnostics) synchronise.  A handle is not thread safe:
 *    use one handle per host thread.
 *  - Host arrays exchanged with `lbm_get_state` / `lbm_set_state` use the reference's
 *    Fortran layout: populations f(0:q-1, 1:nx, 1:ny, 1:nz) with the direction index
 *    fastest, scalar fields T(1:nx, 1:ny, 1:nz) column major (x fastest).
 *  - 2D lattices have dim = 2 and nz = 1.
 */
#ifndef LBM_GPU_H
#define LBM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define LBM_OK            0
#define LBM_ERR_PARAM     1 /* invalid parameters (reference: `stop` after a log line) */
#define LBM_ERR_CUDA      2 /* a CUDA runtime call failed                              */
#define LBM_ERR_OOM       3 /* device allocation refused                               */
#define LBM_ERR_DIVERGED  4 /* non-finite value or rho <= 0 found by a diagnostic      */
#define LBM_ERR_TIMEOUT   5 /* a bounded device-side wait gave up                      */
#define LBM_ERR_STATE     6 /* call not valid for this handle (e.g. precision)         */
#define LBM_ERR_IO        8 /* a file could not be opened, written or parsed            */

/* ---- cell type: CPP switches RayleighBenardCell / SideHeatedCell (3DRB.F90:23-37) --- */
#define LBM_CELL_RB   0 /* heated from below: lengthUnit = ny                            */
#define LBM_CELL_SIDE 1 /* heated side walls: lengthUnit = nx                            */

/* ---- flow boundary per axis: *WallsNoslip / *WallsPeriodicalU (3DRB.F90:14-18) ------ */
#define LBM_BC_NOSLIP   0
#define LBM_BC_PERIODIC 1

/* ---- thermal boundary per axis: *WallsConstT / *Adiabatic / *PeriodicalT ------------ */
#define LBM_BCT_CONST     0 /* low face at Thot, high face at Tcold (anti-bounce-back)   */
#define LBM_BCT_ADIABATIC 1
#define LBM_BCT_PERIODIC  2

/* ---- population storage precision --------------------------------------------------- */
#define LBM_FP64 0 /* plain method: FP64 storage and arithmetic, reference expression order */
#define LBM_FP32 1 /* FP32 storage of deviations from rest weights, FP32 arithmetic          */
#define LBM_FP16 2 /* FP16 storage of deviations from rest weights, FP32 arithmetic          */

/* ---- arithmetic of FP64 handles (lbm_params.arith) ------------------------------------- */
/* LBM_ARITH_REFERENCE: the plain method, the reference's FP64 operations in its expression
 *   order, bit for bit equal to the reference's CPU build (bound by GB300's FP64 pipe).
 * LBM_ARITH_FIXED: the same step to FP64 accuracy on the integer pipes (no counterpart in the
 *   reference).  The fused buffers hold populations as 64-bit fixed-point deviations from
 *   the rest state (units of 2^-60); the moment transforms are exact integer sums and the
 *   relaxation, equilibria, force and 1/rho are 128-bit integer products, each rounded once
 *   below 2^-60.  Results match the reference to rounding (tested: <= 1e-12 relative in the
 *   populations after 1000 steps, <= 1e-10 in Nu, except where the flow amplifies rounding,
 *   where it stays within the distance of the reference's own FMA-contracted build).  The
 *   module arrays, diagnostics, state transfer and restart files are the FP64 handle's; a
 *   restart continues from the FP64 module state.  Two-buffer pattern only; not with
 *   SideHeatedHa. */
#define LBM_ARITH_REFERENCE 0
#define LBM_ARITH_FIXED     1

/* ---- streaming pattern ---------------------------------------------------------------- */
#define LBM_PATTERN_AB 0 /* two population buffers (ping-pong)                              */
#define LBM_PATTERN_AA 1 /* one buffer, in-place even/odd (AA) access pattern               */
/* The in-place pattern gives the same values as the two-buffer pattern, bit for bit, in
 * less than half the device memory (one population array per lattice, which is also the
 * module array).  It keeps no post-collision arrays: LBM_FIELD_F_POST / LBM_FIELD_G_POST
 * and the stage entry points (lbm_collision ... lbm_macroT) return LBM_ERR_STATE, and
 * ensembles take two-buffer handles only. */

/* ---- fields for lbm_get_state / lbm_set_state --------------------------------------- */
#define LBM_FIELD_F       0  /* f(0:q-1,nx,ny,nz), q = 9 (2D) or 19 (3D)                 */
#define LBM_FIELD_G       1  /* g(0:qt-1,nx,ny,nz), qt = 5 (2D) or 7 (3D)                */
#define LBM_FIELD_RHO     2
#define LBM_FIELD_U       3
#define LBM_FIELD_V       4
#define LBM_FIELD_W       5  /* 3D only                                                  */
#define LBM_FIELD_T       6
#define LBM_FIELD_BX_PREV 7
#define LBM_FIELD_BY_PREV 8
#define LBM_FIELD_BZ_PREV 9  /* 3D only                                                  */
#define LBM_FIELD_FX      10 /* 2D only: body force stored by collision (2DRB.F90:718)   */
#define LBM_FIELD_FY      11 /* 2D only                                                  */
#define LBM_FIELD_F_POST  12 /* interior of f_post(0:q-1,0:nx+1,0:ny+1[,0:nz+1])         */
#define LBM_FIELD_G_POST  13 /* interior of g_post                                       */

/* Run parameters: the runtime form of the reference's compile-time `commondata` module
 * (2DRB.F90:48-194, 3DRB.F90:55-187) and of its CPP boundary switches.  Mach follows the
 * reference's definition (tauf = 0.5 + Mach*L*sqrt(3*Pr/Ra)); a free-fall velocity U in
 * lattice units corresponds to Mach = U*sqrt(3). */
typedef struct lbm_params {
    int32_t dim;            /* 2 or 3                                                      */
    int32_t nx, ny, nz;     /* lattice cells; nz = 1 in 2D                                  */
    double  Ra, Pr, Mach;   /* Rayleigh, Prandtl, Mach                                      */
    double  Thot, Tcold;    /* wall temperatures (Tref = (Thot+Tcold)/2)                    */
    int32_t cell;           /* LBM_CELL_RB or LBM_CELL_SIDE                                 */
    int32_t bc_flow[3];     /* per axis x,y,z: LBM_BC_*                                     */
    int32_t bc_thermal[3];  /* per axis x,y,z: LBM_BCT_*                                    */
    int32_t use_g;          /* EnableUseG: M1G heat-flux correction (default 1)            */
    int32_t legacy_thermal; /* EnableLegacyThermalScheme (default 0)                        */
    int32_t precision;      /* LBM_FP64 / LBM_FP32 / LBM_FP16                               */
    int32_t pattern;        /* LBM_PATTERN_AB / LBM_PATTERN_AA                              */
    uint64_t seed;          /* seed of the initial temperature noise                        */
    double  noise_amp;      /* T += noise_amp*(2*xi-1), xi = splitmix64(seed ^ cell) in [0,1) */
    int32_t side_heated_ha; /* SideHeatedHa: magnetic (Lorentz) force, 2D plain FP64 method    */
    int32_t arith;          /* FP64 handles: LBM_ARITH_REFERENCE (0) or LBM_ARITH_FIXED (1)  */
    double  Ha;             /* Hartmann number (2DRB.F90:89, default 20)                     */
    double  phi_deg;        /* field angle in degrees from +x (2DRB.F90:90, default 0)       */
} lbm_params;

/* Derived constants, computed exactly as the reference's `parameter` statements
 * (2DRB.F90:61-115, 3DRB.F90:73-123). */
typedef struct lbm_constants {
    double lengthUnit, Tref, tauf, viscosity, diffusivity, paraA;
    double gBeta, timeUnit, velocityUnit, heatFluxScale, velocityScaleCompare;
    double Snu, Sq, Se, Seps, Spi, Sm;      /* flow MRT rates (2D uses Snu, Sq)         */
    double taug, Qk, Qnu, SG, thermalGeqCoeff, cs2T;
    double omegaT0, omegaT1;                /* thermal weights: rest, moving             */
    double B2sigemarho, phi, sinphi, cosphi; /* SideHeatedHa (2DRB.F90:88-92); sin/cos of phi
                                               as the host's libm gives them                 */
} lbm_constants;

/* Wall Nusselt numbers of RBcalc_Nu_wall_avg (2DRB.F90:2308-2473, 3DRB.F90:2049-2210). */
typedef struct lbm_nu_wall {
    double Nu_hot, Nu_cold, Nu_middle;
    double Nu_hot_max, Nu_hot_max_position;
    double Nu_hot_min, Nu_hot_min_position;
} lbm_nu_wall;

typedef struct lbm_handle lbm_handle;

/* ---- parameters ------------------------------------------------------------------------ */
/* Defaults of a Rayleigh-Benard cell: 2D = 2DRB.F90:11-38 (x periodic, y walls at Thot/Tcold,
 * Ra 5e4, Pr 0.71, Mach 0.1, 320x160); 3D = RB variant of 3DRB.F90:9-47 (no-slip everywhere,
 * adiabatic x/z walls, 120^3, Ra 1e7). */
int lbm_params_default(int dim, lbm_params* out);
/* commondata derivation; replaces the `parameter` block (3DRB.F90:73-123). */
int lbm_derive_constants(const lbm_params* p, lbm_constants* out);

/* ---- lifecycle ------------------------------------------------------------------------- */
/* Allocates every device array the run needs (replaces the `allocate` statements of
 * `initial`, 3DRB.F90:467-473) and a CUDA stream; `device` selects the GPU. */
int lbm_create(const lbm_params* p, int device, lbm_handle** out);
int lbm_destroy(lbm_handle* h);
/* subroutine initial (2DRB.F90:371-663, 3DRB.F90:342-679) with loadInitField = 0. */
int lbm_initial(lbm_handle* h);
const char* lbm_last_error(const lbm_handle* h);
const char* lbm_status_string(int status);
int lbm_get_constants(const lbm_handle* h, lbm_constants* out);
int64_t lbm_itc(const lbm_handle* h);   /* time steps taken since lbm_initial (itc)     */
int lbm_sync(lbm_handle* h);            /* wait for all queued work of the handle       */

/* ---- stage entries: one CUDA kernel per reference subroutine (FP64 handles only) -------- */
int lbm_collision(lbm_handle* h);   /* 2DRB.F90:675-766   3DRB.F90:689-949   */
int lbm_streaming(lbm_handle* h);   /* 2DRB.F90:777-798   3DRB.F90:957-979   */
int lbm_bounceback(lbm_handle* h);  /* 2DRB.F90:811-866   3DRB.F90:987-1058  */
int lbm_macro(lbm_handle* h);       /* 2DRB.F90:878-894   3DRB.F90:1066-1098 */
int lbm_collisionT(lbm_handle* h);  /* 2DRB.F90:906-980   3DRB.F90:1106-1198 */
int lbm_streamingT(lbm_handle* h);  /* 2DRB.F90:993-1014  3DRB.F90:1209-1232 */
int lbm_bouncebackT(lbm_handle* h); /* 2DRB.F90:1026-1107 3DRB.F90:1243-1351 */
int lbm_macroT(lbm_handle* h);      /* 2DRB.F90:1120-1134 3DRB.F90:1362-1381 */

/* ---- fused time stepping ---------------------------------------------------------------- */
/* Advances nsteps time steps (the body of the `do while` loop, 3DRB.F90:225-241) with the
 * fused pull-stream + MRT-collide kernels of the handle's precision, replayed from a
 * captured CUDA graph.  Asynchronous. */
int lbm_step(lbm_handle* h, int64_t nsteps);

/* ---- diagnostics (FP64 reductions on the device; synchronise) --------------------------- */
/* subroutine check: errU = ||u-up||_2/||u||_2, errT = ||T-Tp||_1/||T||_1, then up <- u
 * (2DRB.F90:1213-1260, 3DRB.F90:1475-1528).  Returns LBM_ERR_DIVERGED on a non-finite field. */
int lbm_check(lbm_handle* h, double* errU, double* errT);
/* check with the reference's convergence history (2DRB.F90:1249-1258, 3DRB.F90:1522-1526):
 * lbm_check, then the record (itc, errorU, errorT) appended to <dir>/convergence.plt
 * (3D: convergence3D.plt) and, under the zone lbm_case_tag, to <dir>/convergence_all.plt
 * (3D: convergence_all_3D.plt), then echoed to standard output when echo != 0 (the
 * reference always echoes).  dir NULL or "" = the working directory.  A diverged field is
 * logged and reported as LBM_ERR_DIVERGED. */
int lbm_check_log(lbm_handle* h, const char* dir, int echo, double* errU, double* errT);
/* subroutine append_convergence_tecplot (2DRB.F90:1273-1298, 3DRB.F90:1536-1557): the first
 * call on a handle replaces the file with the header VARIABLES = "itc" "errorU" "errorT",
 * ZONE T="conv" (3D "conv3d"), F=POINT and the record; later calls append the record
 * write(u,'(I12,1X,ES24.16,1X,ES24.16)') (the file must exist, LBM_ERR_IO otherwise). */
int lbm_append_convergence_tecplot(lbm_handle* h, const char* filename, int64_t itc, double errorU, double errorT);
/* subroutine append_convergence_master_tecplot (2DRB.F90:1310-1343, 3DRB.F90:1564-1591): the
 * first call on a handle writes TITLE = "Convergence comparison" (3D: "... 3D") and the
 * VARIABLES line if the file does not exist, then ZONE T="<zone, trailing blanks trimmed>",
 * F=POINT; every call appends the record. */
int lbm_append_convergence_master_tecplot(lbm_handle* h, const char* filename, const char* zone, int64_t itc,
                                          double errorU, double errorT);
/* The caseTag of check: "Ra=<ES10.3E2>,nx=<I0>,ny=<I0>[,nz=<I0>],useG=<T|F>,old=<T|F>"
 * (2DRB.F90:1252-1253, 3DRB.F90:1523-1524). */
int lbm_case_tag(const lbm_handle* h, char* buf, size_t len);
/* subroutine calNuRe: volume Nu = 1 + <v T> L/kappa (RB) or <u T> (side heated) and
 * Re = sqrt(<|u|^2>) L/nu (2DRB.F90:1610-1675, 3DRB.F90:1712-1778). */
int lbm_calNuRe(lbm_handle* h, double* Nu, double* Re);
/* subroutine RBcalc_Nu_global (2DRB.F90:2251-2297, 3DRB.F90:1839-1878). */
int lbm_RBcalc_Nu_global(lbm_handle* h, double* Nu_global);
/* subroutine RBcalc_Nu_wall_avg (2DRB.F90:2308-2473, 3DRB.F90:2049-2210). */
int lbm_RBcalc_Nu_wall_avg(lbm_handle* h, lbm_nu_wall* out);

/* ---- state transfer (Fortran layout, FP64 host arrays) ---------------------------------- */
/* `count` is the number of doubles in `host` and must equal the field's size. */
int lbm_get_state(lbm_handle* h, int field, double* host, size_t count);
int lbm_set_state(lbm_handle* h, int field, const double* host, size_t count);

/* ---- batched form: many lattices in one launch per stage (no counterpart in the
 *      reference, which runs one case per executable) ---------------------------------------
 * An ensemble advances any number of FP32/FP16 handles (one storage precision, any mix of
 * sizes, Ra, Pr, 2D and 3D) with one flow and one thermal launch per step over a packed
 * tile table, replayed from captured CUDA graphs.  Members stay ordinary handles: their
 * diagnostics and state transfer work as usual (the handle's stream waits for the
 * ensemble's work).  A member that is not yet in the fused form (after lbm_initial or
 * lbm_set_state) takes that first step alone at the next lbm_ensemble_step. */
typedef struct lbm_ensemble lbm_ensemble;
int lbm_ensemble_create(int device, lbm_ensemble** out);
int lbm_ensemble_destroy(lbm_ensemble* e);            /* does not destroy the members      */
int lbm_ensemble_add(lbm_ensemble* e, lbm_handle* h);
int lbm_ensemble_remove(lbm_ensemble* e, lbm_handle* h);  /* lbm_destroy also removes     */
int lbm_ensemble_size(const lbm_ensemble* e);
int lbm_ensemble_step(lbm_ensemble* e, int64_t nsteps);
int lbm_ensemble_sync(lbm_ensemble* e);
int lbm_ensemble_get_stream(lbm_ensemble* e, void** stream);
const char* lbm_ensemble_last_error(const lbm_ensemble* e);
/* Tile/block autotuner: times `nsteps` steps of each launch configuration and keeps the
 * fastest (members advance by those steps); outputs may be NULL. */
int lbm_ensemble_autotune(lbm_ensemble* e, int nsteps, int* best_block, int* best_tile, int* best_grid);
/* Launch configuration of the batched step: threads per block (128 or 256), cells per tile
 * (a positive multiple of the block), grid = min(tiles, SMs x grid_mul) with grid_mul in
 * 1..64, and pairs (bit 0: 2D members with even nx take two x-adjacent cells per thread with
 * 2-element vector loads and stores; bit 1: the same for 3D members).  Every configuration
 * gives the same values bit for bit; lbm_ensemble_autotune picks one by timing.
 * LBM_ERR_PARAM for values out of range.  get_launch: outputs may be NULL. */
int lbm_ensemble_configure(lbm_ensemble* e, int block, int tile_cells, int grid_mul, int pairs);
int lbm_ensemble_get_launch(const lbm_ensemble* e, int* block, int* tile_cells, int* grid_mul, int* pairs);
/* Device bytes lbm_create allocates for these parameters (for admission against an HBM
 * budget). */
int lbm_footprint(const lbm_params* p, size_t* bytes);

/* ---- execution options (no counterpart in the reference) --------------------------------
 * LBM_OPT_SINGLE_KERNEL: FP32/FP16 handles advance with one fused kernel per step (1) or
 *   with the two-kernel form (0, default, three times faster on GB300).  Both run the same
 *   arithmetic; T and the thermal populations agree bit for bit, the flow populations to
 *   their last bits (the collision's multiply-adds may fuse differently).  On a 3D FP64
 *   handle with the fixed arithmetic (nx <= 512) it selects the fused pass, which runs the
 *   thermal collision of one step and the flow collision of the next in one launch and sums
 *   each cell's T from pushed values in shared memory (1), or the two-kernel step (0,
 *   default, faster on GB300); both give the same values bit for bit.
 * LBM_OPT_KCHUNK: z planes marched by one block of the fused 3D kernel (default 16).
 * LBM_OPT_PAIRS: the two-kernel FP32/FP16 step moves populations as 2-cell vectors, two
 *   x-adjacent cells per thread (1; used when nx is even) or one cell per thread (0).
 * LBM_OPT_STAGED: the two-kernel FP32/FP16 step stages tiles of x-rows in shared memory
 *   with bulk asynchronous copies (1; used when nx is a multiple of 8; takes precedence
 *   over LBM_OPT_PAIRS) or pulls every value from global memory (0).  A staged kernel
 *   whose bounded wait for its copies gives up sets a device flag: the next lbm_sync or
 *   diagnostic returns LBM_ERR_TIMEOUT.
 * All forms give the same values bit for bit.  Defaults (fastest on GB300): one cell per
 * thread, except two cells per thread for 2D FP32; in the in-place pattern (LBM_PATTERN_AA)
 * the even flow sweep, whose accesses are all the cell's own slots, is always paired when
 * nx is even, and the options select the paired or staged form for the other sweeps.
 * LBM_OPT_FP16_ROUNDING: how FP16 storage rounds the new populations of a step.  Stochastic
 *   (1, default): up with probability equal to the dropped fraction, with random bits keyed
 *   on (step counter, cell, direction), so results are reproducible and the same in every
 *   kernel form and both patterns.  Nearest (0) drops every change smaller than half a unit
 *   in the last place: from a small seed (1e-3 in T) at Ra 1e7 the lattice then never leaves
 *   the conductive state.  Not settable while the handle is in an ensemble. */
#define LBM_OPT_SINGLE_KERNEL 1
#define LBM_OPT_KCHUNK        2
#define LBM_OPT_PAIRS         3
#define LBM_OPT_STAGED        4
#define LBM_OPT_FP16_ROUNDING 5 /* FP16 storage: 1 stochastic rounding (default), 0 nearest */
/* LBM_OPT_HOST_DIRECT: state transfer of an FP64 handle with the layout kernels reading
 *   (bit 0: lbm_set_state) and writing (bit 1: lbm_get_state) the caller's host array
 *   coherently, where the device reports cudaDevAttrPageableMemoryAccess (a GPU attached to a
 *   Grace CPU over NVLink-C2C), instead of staging it through a device buffer with a copy.
 *   Default 1 there (reads; 0 elsewhere): writes into host memory not yet touched fault its
 *   pages in from the GPU side and run slower than a staged copy.  Same values either way;
 *   the host array must stay valid until the call returns (the calls synchronise). */
#define LBM_OPT_HOST_DIRECT   6
/* LBM_OPT_ROWS: FP32/FP16 two-buffer steps launch interior rows (only x can leave the
 *   lattice there: the x rule by selects, no cell-index division) and face rows (the full
 *   boundary rule) as separate kernels (1), or one cell per thread in lattice order (0).  Two
 *   cells per thread, where chosen, takes precedence.  Same values either way. */
#define LBM_OPT_ROWS          7
/* LBM_OPT_WIDE_INDEX: fixed-arithmetic and FP32/FP16 handles index their arrays with 64-bit
 *   integers in every kernel (1), the form lattices of q * ncell >= 2^31 take, or with 32-bit
 *   indices in the main step kernels (the fixed arithmetic's interior rows, the FP16
 *   one-cell kernels and the FP32 thermal kernel, where they measured faster on GB300) where
 *   every index fits (0, default: half the address arithmetic and 32-bit divisions of the
 *   cell index).  Same values either way. */
#define LBM_OPT_WIDE_INDEX    8
int lbm_set_option(lbm_handle* h, int option, int value);

/* ---- measurement hooks (no counterpart in the reference, which times its loop with
 *      CPU_TIME / OMP_get_wtime, 3DRB.F90:222-223, 266-267) -------------------------------- */
/* The handle's CUDA stream (a cudaStream_t), for callers that record their own events. */
int lbm_get_stream(lbm_handle* h, void** stream);
/* Advance nsteps fused steps without graph replay, recording CUDA events around each
 * kernel; returns the mean device time per launch of the flow and thermal kernels. */
int lbm_time_kernels(lbm_handle* h, int64_t nsteps, double* ms_flow, double* ms_thermal);
/* Self-test (no counterpart in the reference): the plain method divides by the reference's
 * integer constants (x/19, x/2394, ...) with a 3-operation correctly rounded sequence; this
 * compares it bitwise with CUDA's IEEE division on n random normal doubles for each of the
 * 19 constants and returns the number of mismatches (expected 0). */
int lbm_selftest_const_division(int64_t n, uint64_t seed, int64_t* mismatches);
/* Self-test (no counterpart in the reference): the plain method computes its products with
 * exact powers of two (2x, x/4, -0.5x, ...) as exponent adds on the integer pipes; this
 * compares those bitwise with the FP64 pipe's products on n generated operands (random,
 * subnormal results included), together with the identity x/(c 2^k) = (x/c) 2^-k for the divisor pairs of the
 * collisions (10/40, 18/36, 18/72, 12/24, 63/252, 6/12, 9/18, 9/36) on normal quotients and
 * the macro step's quotients through one shared correctly rounded reciprocal (x/rho, y/rho,
 * ...) against IEEE division, and returns the number of mismatches (expected 0). */
int lbm_selftest_int_arith(int64_t n, uint64_t seed, int64_t* mismatches);
/* Self-test of failure detection (no counterpart in the reference, which stops the process,
 * 3DRB.F90:1457-1460): on an FP32/FP16 handle, runs the staged kernels' bounded mbarrier
 * wait on a barrier that is armed for bytes no copy delivers (none is issued, so nothing is
 * in flight), for `polls` polls (1 .. 2^24).  The wait gives up and sets the handle's device
 * error flag: the next lbm_sync or diagnostic returns LBM_ERR_TIMEOUT and clears it, and the
 * handle stays usable.  Asynchronous. */
int lbm_selftest_wait_timeout(lbm_handle* h, int64_t polls);

/* ---- allocation-free diagnostic (no counterpart in the reference) -----------------------
 * For callers that cannot let a library call cudaMalloc: programs whose device memory is
 * already owned by their own allocator (the Fortran driver's OpenACC data region or pool,
 * a framework's caching allocator, a server admitting lattices against a fixed HBM
 * budget).  There a library cudaMalloc can fail while the owner's pool still has room,
 * it escapes the owner's accounting, and cudaFree synchronises the whole device.
 *
 * Computes the calNuRe volume averages (Nu = 1 + <v T> L/kappa, or <u T> for a side-heated
 * cell; Re = sqrt(<|u|^2>) L/nu) of caller-provided FP64 device fields of `ncell` values
 * (w = NULL in 2D) on `stream` (a cudaStream_t, NULL = default stream), and returns the
 * two numbers in host memory; the call synchronises that stream.  It allocates nothing:
 * its per-block partial sums live in one fixed array compiled into the library, of
 * 3*LBM_NOALLOC_MAX_BLOCKS+3 doubles (about 29 KB on every GPU that loads the library,
 * held until the process exits).  Lattices larger than LBM_NOALLOC_MAX_CELLS cells are
 * rejected with LBM_ERR_TOO_LARGE before anything is launched.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call outside any stream capture.  That address belongs to the
 * device's primary context: call from that context (the runtime API's), and not after a
 * cudaDeviceReset.  All calls share the array: calls that overlap on the GPU race and must
 * be serialised by the caller.  w = NULL means a 2D field (Re from u and v only); a 3D caller
 * that passes NULL gets Re without the w^2 term and no error.  A non-finite field value
 * gives LBM_ERR_DIVERGED. */
#define LBM_ERR_TOO_LARGE            7
#define LBM_NOALLOC_MAX_BLOCKS       1216  /* partial-sum slots; a call uses min(1216, 4 x SMs) */
#define LBM_NOALLOC_CELLS_PER_BLOCK  65536 /* capacity unit: MAX_CELLS = MAX_BLOCKS x this     */
#define LBM_NOALLOC_MAX_CELLS        (1216LL * 65536LL) /* 79,691,776 cells, e.g. 430^3 */
int lbm_calNuRe_noalloc(const double* u, const double* v, const double* w, const double* T, int64_t ncell,
                        int side_heated, double lengthUnit, double diffusivity, double viscosity,
                        void* stream, double* Nu, double* Re);

/* ---- side-heated cell and mid-line diagnostics ---------------------------------------
 * SideHeatedcalc_Nu_global (2DRB.F90:1686-1734, 3DRB.F90:1789-1828): mean over cells of
 *   [(L/kappa) u (T - Tref) + dT/dx] / (Thot - Tcold), one-sided wall stencils at x faces.
 * SideHeatedcalc_Nu_wall_avg (2DRB.F90:1746-1941, 3DRB.F90:1889-2038): hot (left) wall,
 *   cold (right) wall and x mid-plane means, and the hot wall's extremes along y from the
 *   adiabatic-corner extension and the 5-point least-squares parabola (the fields of
 *   lbm_nu_wall; positions are y).
 * {SideHeated,RB}calc_{u,v,w}mid_max: the largest velocity component on its mid line / plane:
 *   2D (2DRB.F90:2081-2238, 2484-2657): the 5-point parabola through the grid maximum of
 *     u on the vertical mid line (RB: on x = 0.5, interpolated, position folded into the
 *     lower half) or of v on the horizontal mid line; pos1 = position along the line;
 *   3D (3DRB.F90:2345-2518, SideHeated and RB alike): the grid maximum over the mid plane
 *     of the component interpolated to it; pos1/pos2 = the two in-plane coordinates (y,z
 *     for u; x,z for v; x,y for w).
 *   value is in the reference's post-processing scale (times L/kappa); mid = the line /
 *   plane coordinate.  w is 3D only. */
typedef struct lbm_mid_max {
    double value, pos1, pos2, mid;
} lbm_mid_max;
int lbm_SideHeatedcalc_Nu_global(lbm_handle* h, double* Nu_global);
int lbm_SideHeatedcalc_Nu_wall_avg(lbm_handle* h, lbm_nu_wall* out);
int lbm_SideHeatedcalc_umid_max(lbm_handle* h, lbm_mid_max* out);
int lbm_SideHeatedcalc_vmid_max(lbm_handle* h, lbm_mid_max* out);
int lbm_SideHeatedcalc_wmid_max(lbm_handle* h, lbm_mid_max* out);
int lbm_RBcalc_umid_max(lbm_handle* h, lbm_mid_max* out);
int lbm_RBcalc_vmid_max(lbm_handle* h, lbm_mid_max* out);
int lbm_RBcalc_wmid_max(lbm_handle* h, lbm_mid_max* out);

/* ---- snapshot writers and stream-function post-processing ------------------------------
 * output_binary (3DRB.F90:1599-1627, 2DRB.F90:1357-1389): unformatted sequential records
 *   velocityScaleCompare*u, *v, [*w], T, rho to `path`.
 * output_Tecplot (2DRB.F90:1443-1570; 3DRB.F90:1676-1700): the reference's Tecplot binary
 *   files, named as the reference names them from a prefix and a number (12 digits):
 *   2D  <prefix>-<n>.plt (X, Y, U_nd, V_nd, T);
 *   3D  <prefix>-fullField-<n>.plt (3DRB.F90:3018-3099), -midX/-midY/-midZ- mid planes
 *       (2619-2719), -midXpsiVort/-midYpsiVort/-midZpsiVort- stream function and vorticity of
 *       the mid planes (2721-3016).
 * calc_psi_vort_and_output (2D, 2DRB.F90:2657-2780): stream function and vorticity, the
 *   <prefix>-psiVort-<n>.plt file (prefix NULL: no file), psi at the centre by 4x4 Lagrange
 *   interpolation (output_psi_center_abs, 3085-3165), and the largest |psi| on a fine grid of
 *   nFinePerUnit points per unit length with natural splines (calc_psi_absmax_fine_spline,
 *   2873-2998; the reference uses 10000), the fine grid searched on the GPU. */
typedef struct lbm_psi_summary {
    double psi_center, psi_center_abs;         /* coarse-grid Lagrange value at the centre */
    double psi_abs_max, x_at_max, y_at_max;    /* fine-grid maximum of |psi| and position   */
    double psi_center_abs_fine;                /* |psi| at the centre from the splines      */
} lbm_psi_summary;
int lbm_get_params(const lbm_handle* h, lbm_params* out);
int lbm_output_binary(lbm_handle* h, const char* path);
int lbm_output_Tecplot(lbm_handle* h, const char* prefix, int64_t number);
int lbm_calc_psi_vort_and_output(lbm_handle* h, const char* prefix, int64_t number, int nFinePerUnit,
                                 lbm_psi_summary* out);

/* The same writers on host arrays in the Fortran layout (no GPU needed, except the fine-grid
 * search of lbm_psi_absmax_fine_spline, which runs on the current device). */
int lbm_output_binary_host(const char* path, int dim, int nx, int ny, int nz, double velocityScaleCompare,
                           const double* u, const double* v, const double* w, const double* T, const double* rho);
int lbm_tecplot_fields_2d(const char* path, int nx, int ny, double lengthUnit, double velocityScaleCompare,
                          const double* u, const double* v, const double* T);
int lbm_tecplot_full_3d(const char* path, int nx, int ny, int nz, double lengthUnit, const double* u,
                        const double* v, const double* w, const double* T);
int lbm_tecplot_midplane_3d(const char* path, int axis, int nx, int ny, int nz, double lengthUnit,
                            double velocityScaleCompare, const double* u, const double* v, const double* w,
                            const double* T);
int lbm_tecplot_midplane_stream_3d(const char* path, int axis, int nx, int ny, int nz, double lengthUnit,
                                   double velocityScaleCompare, const double* u, const double* v, const double* w);
int lbm_psi_vort_2d(int nx, int ny, double lengthUnit, double velocityScaleCompare, const double* u,
                    const double* v, double* psi, double* vort);
int lbm_tecplot_psi_vort_2d(const char* path, int nx, int ny, double lengthUnit, const double* psi,
                            const double* vort);
int lbm_psi_center_2d(int nx, int ny, double lengthUnit, const double* psi, double* psi_center);
int lbm_psi_absmax_fine_spline(int nx, int ny, double lengthUnit, const double* psi, int nFinePerUnit,
                               double* psi_abs_max, double* x_at_max, double* y_at_max,
                               double* psi_center_abs_fine);

/* Host forms of the convergence-history appenders (no handle, no GPU): `first` stands for
 * the reference's once-per-run flag; dim 2 or 3 picks the zone and title spelling. */
int lbm_append_convergence_tecplot_host(const char* filename, int first, int dim, int64_t itc, double errorU,
                                        double errorT);
int lbm_append_convergence_master_tecplot_host(const char* filename, int first, int dim, const char* zone, int64_t itc,
                                               double errorU, double errorT);
/* One convergence record as the reference writes it, write(u,'(I12,1X,ES24.16,1X,ES24.16)')
 * itc, errorU, errorT, with its newline, into buf (len >= 64). */
int lbm_convergence_line(int64_t itc, double errorU, double errorT, char* buf, size_t len);
/* x in the Fortran edit descriptor ESw.d (e = 0) or ESw.dEe, right-justified in w columns
 * (w asterisks when it does not fit), into buf (len > w). */
int lbm_format_fortran_es(double x, int w, int d, int e, char* buf, size_t len);

/* ---- restart files (backupData, 3DRB.F90:1638-1665 / 2DRB.F90:1402-1430; reload,
 *      3DRB.F90:602-623 / 2DRB.F90:621-637; reconstruct_macro_from_fg,
 *      3DRB.F90:1392-1463 / 2DRB.F90:1144-1200) -----------------------------------------
 * lbm_backupData writes the reference's file: two Fortran unformatted sequential records
 * (gfortran framing: 4-byte length markers, subrecords above 2^31-9 bytes) holding
 * f(alpha,i,j,k) and g(alpha,i,j,k) as FP64, direction outermost and x fastest.  FP32/FP16
 * handles write their populations converted to FP64.  With LBM_BACKUP_CONTINUE the file
 * continues with extra records (a 16 x int64 header, then one record per array in the
 * handle's own storage type) that make the restart bit-continuous: the reference's own
 * reader reads the first two records and never sees them.  The reference's file name is
 * backupFile-<n>.bin (2D) / backupFile3D-<n>.bin (3D); the caller passes the path.
 *
 * lbm_reload replaces the state of a handle (initialised or not, not an ensemble member):
 *   LBM_RELOAD_REFERENCE  read f and g, then rebuild T = sum g, rho, u (3 fixed-point
 *                         passes with F = rho gBeta (T - Tref)), B_prev = u T, 2D Fx/Fy, as
 *                         reconstruct_macro_from_fg does; zero up..Tp and itc.  Not bit-
 *                         continuous: the running solver's u and B_prev used T of the
 *                         previous step.  A cell with rho <= 0 gives LBM_ERR_DIVERGED (the
 *                         reference stops) and leaves the handle uninitialised.
 *   LBM_RELOAD_CONTINUE   read the continuation records too (error LBM_ERR_IO if absent,
 *                         LBM_ERR_PARAM if they were written for another lattice size or
 *                         precision); the next lbm_step continues the saved run bit for bit
 *                         and lbm_itc resumes from the saved count.
 *   LBM_RELOAD_AUTO       CONTINUE when the records are there and match, else REFERENCE. */
#define LBM_BACKUP_REFERENCE 0
#define LBM_BACKUP_CONTINUE  1
#define LBM_RELOAD_REFERENCE 0
#define LBM_RELOAD_CONTINUE  1
#define LBM_RELOAD_AUTO      2
int lbm_backupData(lbm_handle* h, const char* path, int flags);
int lbm_reload(lbm_handle* h, const char* path, int mode);
/* Which form lbm_reload used last on this handle: 0 reference reconstruction, 1 continuation. */
int lbm_reload_form(const lbm_handle* h);

/* Fortran record I/O underneath (host only, no GPU needed).  lbm_fortran_record_write
 * writes one record (append != 0 adds it at the end of the file).  lbm_fortran_record_read
 * reads the record that starts at byte `offset` into `data` (up to `capacity` bytes) and
 * returns its length and the offset of the next record; LBM_ERR_TOO_LARGE if the record
 * is longer than `capacity`.  lbm_fortran_set_subrecord_limit lowers the subrecord size
 * (default and maximum 2^31-9) so the subrecord framing can be exercised on small data. */
int lbm_fortran_record_write(const char* path, int append, const void* data, size_t nbytes);
int lbm_fortran_record_read(const char* path, uint64_t offset, void* data, size_t capacity, size_t* nbytes,
                            uint64_t* next_offset);
int lbm_fortran_set_subrecord_limit(size_t max_subrecord_bytes);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GPU_H */
