/*
 * hydrocuda.h -- C ABI of libhydrocuda.so, a GB300 (sm_103a) implementation of
 * hydro-cl-lua's finite-volume Euler update: ghost-cell boundary fill, PLM
 * reconstruction ("plm cons", "plm prim", "plm athena") with the reference's
 * slope limiters, the Roe flux on the Euler eigen-decomposition (optionally
 * flux-limited) or the HLL / Rusanov / HLLC fluxes, calcDerivFromFlux, the CFL
 * calcDT min-reduction, constrainU, and the explicit forward-Euler and
 * Runge-Kutta integrators; batched solving and serving; initial conditions
 * built on the device; display variables and headless views.
 *
 * Plain C99; no callbacks; no library types in the signatures.  Every entry
 * point returns 0 (HC_OK) or a negative HC_ERR_* code; hc_last_error() gives a
 * thread-local message for the last failure on the calling thread.  The
 * caller owns every host array passed in; nothing is retained after return.
 * Device memory is owned by the library behind opaque handles.  A handle is
 * used from one host thread at a time.
 *
 * Reference interfaces replaced (paths within hydro-cl-lua):
 *   solver construction   hydro/solver/solverbase.lua:324-398, gridsolver.lua:60-136,
 *                         fvsolver.lua:28-31, 201-211 (the solver args table)
 *   resetState            hydro/solver/solverbase.lua:2094-2114
 *   boundary              hydro/solver/gridsolver.lua:1316-1320 (kernels 1070-1213)
 *   constrainU            hydro/solver/solverbase.lua:2116-2128, hydro/eqn/euler.cl:697-717
 *   calcDT                hydro/solver/solverbase.lua:3004-3024, hydro/eqn/cl/calcDT.cl:38-73
 *   step / integrate      hydro/solver/solverbase.lua:3193-3238, hydro/int/fe.lua:33-49,
 *                         hydro/int/rk.lua:98-218
 *   update                hydro/solver/solverbase.lua:3026-3190
 *   App exit loop         hydro/app.lua:1573-1600 (t >= exitTime checked before stepping)
 *   UBuf readback         hydro/solver/gridsolver.lua:1337-1366 (UBufObj:toCPU)
 *   display variables     hydro/solver/solverbase.lua:1950-2065, 2871-2994
 *   views                 hydro/draw/2d_heatmap.glsl, volumetric.glsl, vector_lic.glsl
 */
#ifndef HYDROCUDA_H
#define HYDROCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HC_VERSION_MAJOR 0
#define HC_VERSION_MINOR 3

/* return codes */
#define HC_OK               0
#define HC_ERR_INVALID     -1   /* bad argument or unsupported option combination */
#define HC_ERR_CUDA        -2   /* a CUDA runtime call failed */
#define HC_ERR_NOMEM       -3   /* device or host allocation failed */
#define HC_ERR_BUDGET      -4   /* admission would exceed the batch's HBM budget */
#define HC_ERR_NO_SLOT     -5   /* every batch slot is in use */
#define HC_ERR_NONFINITE   -6   /* a solve produced a non-finite dt or state */
#define HC_ERR_TIMEOUT     -7   /* a bounded device wait ran out */
#define HC_ERR_STATE       -8   /* call not valid in the handle's current state */

/* boundary names (gridsolver.lua:617-860); the sphere / cylinder ones need
 * curvilinear coordinates: not provided */
#define HC_BOUNDARY_NONE      0
#define HC_BOUNDARY_PERIODIC  1
#define HC_BOUNDARY_MIRROR    2
#define HC_BOUNDARY_FREEFLOW  3
#define HC_BOUNDARY_LINEAR    4   /* ghost = 2 U[i1] - U[i2], ghosts filled outward (gridsolver.lua:783-813) */
#define HC_BOUNDARY_QUADRATIC 5   /* ghost = 3 U[i1] - 3 U[i2] + U[i3] (gridsolver.lua:815-858) */
#define HC_BOUNDARY_FIXED     6   /* Dirichlet: every ghost cell of the side holds the constant state
                                     fixed_cons (BoundaryFixed, gridsolver.lua:746-765, whose fixedCode
                                     writes one constant cons_t, as the square cavity's does,
                                     hydro/init/euler.lua:1856-1875) */
#define HC_NUM_BOUNDARIES     7

/* limiter table, in the order of hydro/app.lua:614-635 (reference index - 1);
 * HC_LIMITER_DONOR_CELL as flux limiter means "no flux limiter" */
#define HC_LIMITER_DONOR_CELL        0
#define HC_LIMITER_LAX_WENDROFF      1
#define HC_LIMITER_BEAM_WARMING      2
#define HC_LIMITER_FROMM             3
#define HC_LIMITER_CHARM             4
#define HC_LIMITER_HCUS              5
#define HC_LIMITER_HQUICK            6
#define HC_LIMITER_KOREN             7
#define HC_LIMITER_MINMOD            8
#define HC_LIMITER_OSHKER            9
#define HC_LIMITER_OSPRE            10
#define HC_LIMITER_SMART            11
#define HC_LIMITER_SWEBY            12
#define HC_LIMITER_UMIST            13
#define HC_LIMITER_VAN_ALBADA_1     14
#define HC_LIMITER_VAN_ALBADA_2     15
#define HC_LIMITER_VAN_LEER         16
#define HC_LIMITER_MONOTIZED_CENTRAL 17
#define HC_LIMITER_SUPERBEE         18
#define HC_LIMITER_BARTH_JESPERSEN  19
/* Not a row of the reference's table: the van Leer form the reference keeps
 * beside its table entry as a comment (hydro/app.lua:631),
 * (r + |r|) / (1 + |r|).  It equals the table's max(0, r) * 2 / (1 + r) for
 * every r except r = -1, where the table's expression divides 0 by 0. */
#define HC_LIMITER_VAN_LEER_ABS     20
#define HC_NUM_LIMITERS             21

/* usePLM (hydro/solver/plm.cl) */
#define HC_RECON_NONE                0   /* usePLM = nil: interface states are the cell states */
#define HC_RECON_PIECEWISE_CONSTANT  1   /* "piecewise constant" */
#define HC_RECON_PLM_CONS            2   /* "plm cons" */
#define HC_RECON_PLM_PRIM            3   /* "plm prim" (plm.cl:191-253) */
#define HC_RECON_PLM_ATHENA          4   /* "plm athena" (plm.cl:782-879, with its L/R assignment) */
#define HC_NUM_RECONS                5

/* interface flux (the modules of hydro/flux); the flux limiter applies to Roe only
 * (fvsolver.lua:62-64) */
#define HC_FLUX_ROE      0   /* "roe" (roe.cl) */
#define HC_FLUX_HLL      1   /* "hll", waves 'Davis direct bounded' (hll.cl) */
#define HC_FLUX_RUSANOV  2   /* "rusanov" (rusanov.cl) */
#define HC_FLUX_HLLC     3   /* "euler-hllc" (euler-hllc.cl), waves as hll */
#define HC_NUM_FLUXES    4

/* euler-hllc's hllcMethod (2012 Toro): HC_HLLC_DEFAULT is the reference's
 * default, its method 2 */
#define HC_HLLC_DEFAULT  0
#define HC_HLLC_METHOD_0 1   /* Toro eqns 38-39 */
#define HC_HLLC_METHOD_1 2   /* variation 1 */
#define HC_HLLC_METHOD_2 3   /* variation 2 */

/* explicit integrators (hydro/int/all.lua) */
#define HC_INT_FORWARD_EULER   0
#define HC_INT_RK2             1   /* "Runge-Kutta 2" (midpoint) */
#define HC_INT_RK2_HEUN        2
#define HC_INT_RK2_RALSTON     3
#define HC_INT_RK3             4
#define HC_INT_RK4             5
#define HC_INT_RK4_38          6   /* "Runge-Kutta 4, 3/8ths rule" */
#define HC_INT_RK2_TVD         7
#define HC_INT_RK2_NONTVD      8
#define HC_INT_RK3_TVD         9
#define HC_INT_RK4_TVD        10
#define HC_INT_RK4_NONTVD     11
#define HC_NUM_INTEGRATORS    12

/* arithmetic forms */
#define HC_F64_PLAIN   0   /* kernel-for-kernel FP64 form of the reference, array-of-structs */
#define HC_F64_FUSED   1   /* fused stage kernel, structure-of-arrays, FP64 */
#define HC_F32_FUSED   2   /* fused stage kernel, FP32 bulk; FP64 dt reduction, time and sums */

/* host array layouts for state I/O.  Cells in x-fastest order.
 * AOS6_F64: cons_t {rho, m.x, m.y, m.z, ETotal, ePot} as 6 doubles per cell
 * SOA5_F64: 5 planes of doubles (rho, m.x, m.y, m.z, ETotal); ePot is 0
 * SOA5_F32: 5 planes of floats */
#define HC_LAYOUT_AOS6_F64  0
#define HC_LAYOUT_SOA5_F64  1
#define HC_LAYOUT_SOA5_F32  2

/* The solver args table (solverbase.lua:324-338; gridsolver.lua:98-104) as a struct. */
typedef struct hc_solver_desc {
    int    dim;              /* 1, 2 or 3 */
    int    n[3];             /* gridSize without ghosts; unused axes ignored */
    double mins[3];          /* domain; unused axes keep their extent for grid_dx */
    double maxs[3];
    int    boundary[6];      /* xmin xmax ymin ymax zmin zmax, HC_BOUNDARY_* */
    int    flux_limiter;     /* HC_LIMITER_* (Roe flux limiter; donor cell = off) */
    int    recon;            /* HC_RECON_* */
    int    slope_limiter;    /* HC_LIMITER_* (used by PLM) */
    int    integrator;       /* HC_INT_* */
    int    precision;        /* HC_F64_PLAIN | HC_F64_FUSED | HC_F32_FUSED */
    double gamma;            /* heatCapacityRatio, reference default 7/5 */
    double rho_min;          /* reference default 1e-7 */
    double p_min;            /* reference default 1e-7 */
    double cfl;              /* reference default .5 */
    double fixed_dt;         /* > 0: useFixedDT with this dt; <= 0: CFL dt */
    int    flux;             /* HC_FLUX_* (0 = roe) */
    int    hllc_method;      /* HC_HLLC_* (euler-hllc only) */
    /* Roe only: useEntropyFluxFix (hydro/flux/roe.lua:10-16, roe.cl:83-101),
     * off by default: where |lambda| < factor * Cs, lambda becomes
     * sign(lambda) (lambda^2 / (factor Cs) + factor Cs) / 2 */
    int    entropy_fix;      /* 0: off, 1: on */
    int    reserved0;
    double entropy_fix_factor;   /* entropyFluxFixLimitingFactor; the reference's default is .2 */
    /* the ghost cells' conserved state (rho, m.x, m.y, m.z, ETotal) of each
     * side whose boundary is HC_BOUNDARY_FIXED, in boundary[]'s order (ePot 0) */
    double fixed_cons[6][5];
} hc_solver_desc;

/* Initial conditions generated on the device (the reference builds every
 * initial state with its initCond kernel, solverbase.lua:2094-2136).  p[] by
 * kind (hc_init_defaults fills the defaults):
 *   SOD               rhoL, PL, rhoR, PR; left where x < mid on every active axis
 *                     (hydro/init/euler.lua:742-752)
 *   BLAST             radius, Pin, Pout, rho; P = Pin where |x| < radius
 *   QUADRANT          4 x (rho, vx, vy, P) in the reference's quadrant order
 *                     (+x+y, -x+y, -x-y, +x-y) (hydro/init/euler.lua:249-283); 2D
 *   KELVIN_HELMHOLTZ  noise; |y| < .25: rho 2, vx .5, else rho 1, vx -.5; P 2.5;
 *                     vy = noise * U(-1, 1) from SplitMix64(seed), one draw per
 *                     cell in x-fastest order; 2D
 * The states equal, bit for bit, the host generators of the Python binding. */
#define HC_INIT_SOD               0
#define HC_INIT_BLAST             1
#define HC_INIT_QUADRANT          2
#define HC_INIT_KELVIN_HELMHOLTZ  3

typedef struct hc_init {
    int                kind;     /* HC_INIT_* */
    int                reserved;
    unsigned long long seed;     /* KELVIN_HELMHOLTZ */
    double             p[16];
} hc_init;

typedef struct hc_context hc_context;
typedef struct hc_solver  hc_solver;
typedef struct hc_batch   hc_batch;

/* ---- library / context ------------------------------------------------ */

/* Version string "major.minor". */
const char* hc_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* hc_last_error(void);
/* Measurement aid (no counterpart in the reference): the current device's
 * fused multiply-add throughput in TFLOP/s (2 flops per FMA), from a kernel of
 * independent FMA chains; precision HC_F32_FUSED (FP32) or HC_F64_FUSED /
 * HC_F64_PLAIN (FP64). */
int hc_measure_fma(int precision, double* tflops);
/* Number of visible CUDA devices. */
int hc_device_count(int* count);
/* One context per device; owns the streams the handles below use.
   hc_context_destroy releases the caller's reference: the context itself
   lives on until every solver and batch made on it is destroyed too. */
int hc_context_create(int device, hc_context** out);
int hc_context_destroy(hc_context* ctx);
/* Pinned host memory for fast state transfers (optional). */
int hc_host_alloc(size_t bytes, void** out);
int hc_host_free(void* p);
/* The default parameters of an initial condition. */
int hc_init_defaults(int kind, hc_init* out);

/* ---- single solver (FiniteVolumeSolver with flux='roe', eqn='euler') ---- */

/* Validates the descriptor and allocates device state.  Replaces the
 * solver class construction, solverbase.lua:351-398. */
int hc_solver_create(hc_context* ctx, const hc_solver_desc* desc, hc_solver** out);
int hc_solver_destroy(hc_solver* s);
/* resetState after applyInitCond (solverbase.lua:2094-2114): writes the
 * interior conserved state, fills the ghosts, applies constrainU, sets t = 0. */
int hc_solver_reset_state(hc_solver* s, const void* cons, int layout);
/* resetState with the initial condition built on the device (applyInitCond,
 * solverbase.lua:2130-2136): no host array, no upload. */
int hc_solver_init_state(hc_solver* s, const hc_init* init);
/* Raw state I/O.  with_ghosts = 1 reads/writes the reference's whole UBuf,
 * numGhost = 2 layers included (AOS6_F64 only); 0 the interior only.  The
 * plain form holds the UBuf itself; the fused forms return their interior
 * with the ghosts filled by the boundary rules (gridsolver.lua:638-780), and
 * take the interior of a UBuf written to them. */
int hc_solver_set_state(hc_solver* s, const void* cons, int layout, int with_ghosts);
int hc_solver_get_state(hc_solver* s, void* cons, int layout, int with_ghosts);
/* GridSolver:boundary() (gridsolver.lua:1316). */
int hc_solver_boundary(hc_solver* s);
/* SolverBase:constrainU() (solverbase.lua:2116), boundary included. */
int hc_solver_constrain_u(hc_solver* s);
/* SolverBase:calcDT() (solverbase.lua:3004): cfl * min over cells, or fixed_dt. */
int hc_solver_calc_dt(hc_solver* s, double* dt);
/* SolverBase:step(dt) (solverbase.lua:3193): one integrator step. */
int hc_solver_step(hc_solver* s, double dt);
/* SolverBase:update() (solverbase.lua:3026): calcDT, step, t += dt, boundary. */
int hc_solver_update(hc_solver* s, double* dt_out);
/* The fused forms' stage-kernel schedule for this solver's grid, chosen as
 * hc_batch_autotune chooses it (every schedule gives the same bits), without
 * advancing the solve: its state and time are as before the call.  No-op on
 * the plain form.  No counterpart in the reference. */
int hc_solver_autotune(hc_solver* s, const char* cache_path);
/* ---- one grid cut into slabs across devices or ranks --------------------------
 *
 * The reference's multi-device solver (hydro/solver/choppedup.lua) cuts a
 * grid into blocks, copies the ghost layers between neighbouring blocks
 * (syncBorders, choppedup.lua:193-230) and takes the minimum of the blocks' dt
 * on the host (Chopped:update, choppedup.lua:344-400), once per update.  These
 * calls let the same happen per Runge-Kutta stage, which is what reproduces
 * the single-domain result for every integrator: give each slab's solver the
 * boundary "none" on its internal faces, take the ranks' minimum of
 * hc_solver_calc_dt, then for each stage exchange the slabs next to the
 * internal faces and run the stage.  Fused forms only (HC_ERR_INVALID on the
 * plain form, which steps whole updates).
 *
 * hc_solver_stage runs the next stage of the update with the update's dt (the
 * first call sets up the step, the last one completes it; t is not advanced,
 * as with hc_solver_step); hc_solver_step / hc_solver_update refuse while an
 * update is part done (HC_ERR_STATE).  hc_solver_num_stages gives the
 * integrator's stage count.  hc_solver_get_slab copies the two interior
 * layers next to face (axis 0..dim-1, side 0: min, 1: max) of the state the
 * next stage reads to the host; hc_solver_set_slab writes the two ghost
 * layers beyond that face.  Both as cons_t (6 doubles per cell, ePot 0),
 * x-fastest over the two-layer slab (extent 2 along `axis`, the interior
 * extents along the others). */
int hc_solver_stage(hc_solver* s, double dt);
int hc_solver_num_stages(hc_solver* s, int* n);
int hc_solver_get_slab(hc_solver* s, int axis, int side, double* out);
int hc_solver_set_slab(hc_solver* s, int axis, int side, const double* in);
/* The App loop: while t < t_end and steps < max_steps, update().  The test is
 * made before each update, so the final step overshoots t_end (app.lua:1590). */
int hc_solver_run_until(hc_solver* s, double t_end, long long max_steps, long long* steps_done);
int hc_solver_get_time(hc_solver* s, double* t);
int hc_solver_set_time(hc_solver* s, double t);
/* Kahan-compensated FP64 sums of rho, m.x, m.y, m.z, ETotal times cell volume
 * over the interior. */
int hc_solver_conservation(hc_solver* s, double sums[5]);
/* HC_OK, or the first error a kernel recorded (HC_ERR_NONFINITE, HC_ERR_TIMEOUT). */
int hc_solver_status(hc_solver* s);

/* ---- batched, continuously admitted solves ------------------------------ */

typedef struct hc_batch_desc {
    int    precision;        /* HC_F32_FUSED or HC_F64_FUSED */
    int    flux_limiter;     /* shared by every instance of the batch */
    int    recon;
    int    slope_limiter;
    int    integrator;
    int    max_slots;        /* slot table size */
    size_t hbm_budget;       /* bytes of device state the batch may hold */
    int    flux;             /* HC_FLUX_* shared by every instance (0 = roe) */
    int    hllc_method;      /* HC_HLLC_* (euler-hllc only) */
} hc_batch_desc;

typedef struct hc_done {
    int                slot;
    int                status;   /* HC_OK or HC_ERR_NONFINITE */
    unsigned long long tag;
    long long          steps;
    double             t;
} hc_done;

typedef struct hc_batch_stats {
    int       active;            /* instances still stepping */
    int       occupied;          /* slots holding a result or a live instance */
    size_t    bytes_in_use;      /* device state bytes charged to the budget */
    long long tiles;             /* tiles in the current work list */
    long long cells;             /* interior cells of live instances */
    int       n_stages;          /* stage launches per update and dimension */
    int       tile[3][3];        /* tile shape (x, y, z) in use per dimension 1..3 */
    int       schedule[3];       /* stage-kernel schedule in use per dimension (hc_batch_set_schedule's variant) */
    int       marching[3];       /* 1: that schedule's kernel marches strips (2D) or tiles (3D) along the
                                    grid instead of loading tiles */
} hc_batch_stats;

int hc_batch_create(hc_context* ctx, const hc_batch_desc* desc, hc_batch** out);
int hc_batch_destroy(hc_batch* b);
/* Admits one instance: validates it against the batch's shared scheme,
 * charges its state bytes to the HBM budget (HC_ERR_BUDGET if over) and takes
 * a free slot (HC_ERR_NO_SLOT if none), uploads the interior conserved state,
 * applies resetState, computes its first dt.  The instance then advances with
 * every hc_batch_step until t >= t_end or max_steps updates. */
int hc_batch_admit(hc_batch* b, const hc_solver_desc* desc, const void* cons, int layout,
                   double t_end, long long max_steps, unsigned long long tag, int* slot);
/* hc_batch_admit with the initial condition built on the device.  Reads no
 * host buffer after return, so it does not wait: the set-up launches queue
 * behind any hc_batch_step_async in flight. */
int hc_batch_admit_init(hc_batch* b, const hc_solver_desc* desc, const hc_init* init,
                        double t_end, long long max_steps, unsigned long long tag, int* slot);
/* `count` hc_batch_admit calls in one: instance k from descs[k], cons[k],
 * t_end[k], max_steps[k], tags[k] (t_end, max_steps, tags may be NULL: +inf,
 * no limit, k), all in `layout`.  Every instance is checked first; the
 * descriptors of the accepted ones are uploaded together and their states set
 * up by batched launches (one per grid dimension and 120 instances), queued
 * back to back and waited for once.  A buffer in page-locked
 * host memory (hc_host_alloc, cudaHostRegister) is read in place by its
 * set-up kernel over the host link; other buffers go through a staging copy.
 * Stops at the first refusal or error and returns it; *n_admitted = the
 * instances admitted before it (they stay admitted), slots[k] their slots, -1
 * for the rest. */
int hc_batch_admit_many(hc_batch* b, int count, const hc_solver_desc* descs, const void* const* cons, int layout,
                        const double* t_end, const long long* max_steps, const unsigned long long* tags,
                        int* slots, int* n_admitted);
/* Advances every live instance by up to `steps` updates (each instance with its
 * own CFL dt), in batched launches.  *n_active = instances still stepping. */
int hc_batch_step(hc_batch* b, int steps, int* n_active);
/* hc_batch_step without the wait (no counterpart in the reference: the serving
 * loop's tick): the updates are queued on the batch's stream and the call
 * returns, so the host admits, polls or fetches while they run.  Errors of the
 * queued work surface at the next hc_batch_wait or hc_batch_step. */
int hc_batch_step_async(hc_batch* b, int steps);
/* Waits for the work queued by hc_batch_step_async (and any admission queued
 * after it); *n_active (may be NULL) as for hc_batch_step. */
int hc_batch_wait(hc_batch* b, int* n_active);
/* Measurement form of hc_batch_step: the same launches, issued directly (not
 * from the captured graph) with CUDA events around every stage kernel on the
 * batch's stream.  Adds the elapsed milliseconds of stage s (all dimensions,
 * summed over the steps) to stage_ms[s] for s < n_stage_ms, and of the whole
 * span to *total_ms. */
int hc_batch_step_timed(hc_batch* b, int steps, double* stage_ms, int n_stage_ms, double* total_ms);
/* Lists finished instances not yet reported (at most cap). */
int hc_batch_poll(hc_batch* b, hc_done* out, int cap, int* n_out);
/* Lists every occupied slot, finished or not, in slot order (at most cap):
 * its status so far, tag, updates done and time.  Reports nothing as
 * finished (hc_batch_poll still does).  No counterpart in the reference: the
 * batch's progress report. */
int hc_batch_list(hc_batch* b, hc_done* out, int cap, int* n_out);
/* Copies a slot's interior state to the host. */
int hc_batch_fetch(hc_batch* b, int slot, void* cons, int layout);
/* `count` hc_batch_fetch calls in one (slot slots[k] into cons[k], all in
 * `layout`): batched gather launches (one per grid dimension and 120 slots),
 * queued back to back and waited for once; a page-locked buffer is written in
 * place by the gather kernel.  Checks every slot before copying anything. */
int hc_batch_fetch_many(hc_batch* b, int count, const int* slots, void* const* cons, int layout);
/* Frees a slot and returns its bytes to the budget. */
int hc_batch_retire(hc_batch* b, int slot);
int hc_batch_stats_get(hc_batch* b, hc_batch_stats* out);
int hc_batch_conservation(hc_batch* b, int slot, double sums[5]);
/* Times the candidate schedules (tile shape, segment length, threads) of the
 * stage kernel on the batch's live instances and keeps the fastest; reads /
 * writes the choice from / to cache_path when not NULL.  Timing runs whole
 * steps (4 per candidate): the live solves advance by those steps, exactly as
 * hc_batch_step would advance them (every schedule gives the same bits). */
int hc_batch_autotune(hc_batch* b, const char* cache_path);
/* Pins the schedule (tile shape, segment length, threads, lanes: the
 * `variant` numbers of the autotuner's log) of the stage kernel for grids of
 * dimension `dim`.  HC_ERR_INVALID if this scheme has no such schedule.
 * A marching schedule's segments are shortened when its items would fill
 * fewer than two rounds of the launch's resident warps (2D) or CTAs (3D), as
 * for one small grid; HC_MARCH_SEGMENT=<rows> in the environment when the
 * batch is created fixes them at min(rows, the schedule's) instead. */
int hc_batch_set_schedule(hc_batch* b, int dim, int variant);

/* ---- headless visualisation ----------------------------------------------------
 *
 * The reference's display variables of the Euler equations
 * (hydro/eqn/euler.lua:240-260, the state fields of eqn.lua:913-915; vector
 * variables by component and magnitude), evaluated on the device in double
 * with the reference's expressions. */
#define HC_DISPLAY_RHO              0   /* U rho */
#define HC_DISPLAY_MX               1   /* U m x */
#define HC_DISPLAY_MY               2
#define HC_DISPLAY_MZ               3
#define HC_DISPLAY_M_MAG            4   /* U m mag */
#define HC_DISPLAY_ETOTAL           5   /* U ETotal */
#define HC_DISPLAY_EPOT             6   /* U ePot */
#define HC_DISPLAY_VX               7   /* U v x */
#define HC_DISPLAY_VY               8
#define HC_DISPLAY_VZ               9
#define HC_DISPLAY_V_MAG           10
#define HC_DISPLAY_P               11
#define HC_DISPLAY_EINT_SPECIFIC   12   /* eInt */
#define HC_DISPLAY_EKIN_SPECIFIC   13   /* eKin */
#define HC_DISPLAY_ETOTAL_SPECIFIC 14   /* eTotal */
#define HC_DISPLAY_EINT            15   /* EInt */
#define HC_DISPLAY_EKIN            16   /* EKin */
#define HC_DISPLAY_EPOT_VOLUME     17   /* EPot */
#define HC_DISPLAY_S               18
#define HC_DISPLAY_H               19
#define HC_DISPLAY_H_SPECIFIC      20   /* h */
#define HC_DISPLAY_HTOTAL          21
#define HC_DISPLAY_HTOTAL_SPECIFIC 22   /* hTotal */
#define HC_DISPLAY_CS              23   /* speed of sound */
#define HC_DISPLAY_MACH            24   /* Mach number */
#define HC_DISPLAY_TEMPERATURE     25
#define HC_NUM_DISPLAY_VARS        26

/* calcDisplayVarToBuffer (solverbase.lua:1950-2065): `var` at every cell of
 * the grid, ghosts included (numGhost = 2 on each active axis, x fastest),
 * into `out` (host doubles).  A ghost cell shows its nearest interior cell,
 * or 0 when zero_border is set. */
int hc_solver_display(hc_solver* s, int var, int zero_border, double* out);
/* calcDisplayVarRangeAndAvgAndStdDev (solverbase.lua:2871-2994): out = {min,
 * max, mean, standard deviation}; min and max over the grid (equal to those
 * of the interior, ghosts showing interior cells), mean and deviation over
 * the interior cells. */
int hc_solver_display_range(hc_solver* s, int var, double out[4]);

/* Views: the shader arithmetic of hydro/draw/2d_heatmap.glsl, volumetric.glsl
 * and vector_lic.glsl, rendered by CUDA kernels into an RGBA8 image (row 0 at
 * the bottom, as glReadPixels returns it); no graphics API is involved. */
#define HC_RENDER_HEATMAP  0   /* a slice of `var` through the palette */
#define HC_RENDER_VOLUME   1   /* a ray march through a 3D grid */
#define HC_RENDER_LIC      2   /* line-integral convolution of the velocity, coloured by |v| */
#define HC_RENDER_SLICES   3   /* 3d_slice.glsl: a stack of slices through a 3D grid, blended back to front */

/* the palettes written out in hydro/draw/palette.lua, in its order */
#define HC_PALETTE_WHITE_RAINBOW_BLACK 0
#define HC_PALETTE_STRIPES             1
#define HC_PALETTE_BLUE                2
#define HC_PALETTE_PARAVIEW            3   /* paraview-red-grey-blue */

typedef struct hc_render {
    int mode;                 /* HC_RENDER_* */
    int var;                  /* HC_DISPLAY_* (heat map and volume) */
    int width, height;        /* pixels */
    int palette;              /* HC_PALETTE_* */
    int use_log;              /* logarithmic palette mapping (draw.glsl:52-71) */
    double value_min, value_max;   /* mapped onto the palette; min >= max: the variable's range */
    double bbox[4];           /* heat map / LIC: chart rectangle x1, y1, x2, y2 the image covers;
                                 all equal: the domain */
    double slice_angle[4];    /* displaySliceAngle quaternion (x, y, z, w) */
    double fixed_z;           /* displayFixed.y: chart z of the slice before the rotation */
    double eye[3];            /* volume: camera position (chart coordinates), looking at the domain's centre */
    double fov_y;             /* volume: vertical field of view, degrees */
    double alpha, alpha_gamma, num_isobars;   /* volume: volumetric.glsl uniforms */
    int max_iter;             /* volume: maxiter */
    int use_isobars, use_lighting;
    int lic_iter;             /* LIC: integralMaxIter */
    int noise_size;           /* LIC: noise texture edge (drawVectorLICNoiseSize) */
    int reserved;
    unsigned long long noise_seed;   /* LIC: SplitMix64 seed of the noise texture */
    int slice_axis;           /* slices: view axis 0..2 looking towards +axis, 3..5 towards -axis */
    int num_slices;           /* slices: numSlices (the stack has num_slices + 1 slices) */
} hc_render;

/* The reference's defaults for a view (palette 1, identity slice rotation,
 * integralMaxIter 10, noise 1024^2, 255 slices, alpha .15) and a 512 x 512 image. */
int hc_render_defaults(int mode, hc_render* out);
/* Renders the solver's state into rgba (host, width * height * 4 bytes). */
int hc_solver_render(hc_solver* s, const hc_render* r, unsigned char* rgba);

/* ---- calcDT without allocation ---------------------------------------------
 *
 * No counterpart in the reference.  For callers that must not allocate device
 * memory when they need a time step: code whose device memory belongs to an
 * outside allocator (a framework's caching allocator, a fixed arena handed to
 * the library), and loops that cannot take cudaMalloc's implicit device-wide
 * synchronisation or its unbounded time.  The same calcDT as
 * hc_solver_calc_dt on the plain FP64 form: `state` is that form's UBuf in
 * device memory (cons_t as 6 doubles per cell, x-fastest, numGhost = 2 ghost
 * layers on each active axis); cfl * min (or fixed_dt when > 0) is written to
 * the double at `dt_out` in device memory, on `stream` (a cudaStream_t; NULL =
 * the legacy default stream).  Only the descriptor's dim, n, mins, maxs, gamma,
 * rho_min, p_min, cfl and fixed_dt are read, and they are checked as
 * hc_solver_create checks them.  It allocates nothing: the reduction's block
 * minima go to a fixed array inside the library (512 KiB, held on every device
 * that loads the library until the process exits), which caps the grid at
 * HC_NOALLOC_MAX_CELLS cells including ghosts; larger grids return
 * HC_ERR_INVALID.  The first call on a device looks up that array's address
 * (with the device current), so make it before any stream capture; the
 * address is kept for the process's life, so the entry point is not for use
 * after a cudaDeviceReset.  Every call shares the array: calls whose kernels
 * may overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Nothing in the array needs clearing between
 * calls. */
#define HC_NOALLOC_MAX_CELLS (1 << 24)
int hc_calc_dt_noalloc(const hc_solver_desc* desc, const double* state, double* dt_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HYDROCUDA_H */
