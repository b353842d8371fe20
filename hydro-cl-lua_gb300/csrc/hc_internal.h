// hc_internal.h -- shared definitions of libhydrocuda (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/hydrocuda.h"

namespace hc {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define HC_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t hc_e_ = (call);                                            \
        if (hc_e_ != cudaSuccess) return ::hc::cuda_fail(hc_e_, #call);        \
    } while (0)

#define HC_CHECK(call)                                                         \
    do {                                                                       \
        int hc_r_ = (call);                                                    \
        if (hc_r_ != HC_OK) return hc_r_;                                      \
    } while (0)

// Device error flags written by kernels (bounded waits, non-finite results).
enum DeviceStatus : int {
    DEV_OK = 0,
    DEV_NONFINITE = 1,
    DEV_TIMEOUT = 2,
};

// ---------------------------------------------------------------------------
// Runge-Kutta tables (hydro/int/all.lua:10-155); index 0 = forward Euler.
// ---------------------------------------------------------------------------

struct RKTable {
    int order;            // number of stages (forward Euler: 1)
    double alpha[4][4];   // alpha[i-1][k-1]: u^(i) = sum_k alpha u^(k) + dt beta L(u^(k))
    double beta[4][4];
};
const RKTable& rk_table(int integrator);

// The stage plan turns a table into fused stage launches with buffer reuse.
struct StageTerm { int buf; double coef; };
struct StagePlan {
    int index;                    // stage number within the step (0-based)
    int in_buf;                   // u^(i-1), read with halo
    int out_buf;                  // u^(i)
    int n_alpha;                  // alpha terms, k ascending
    StageTerm alpha[4];           // buf = state buffer index (may equal in_buf)
    int n_beta;                   // stored-derivative terms, k ascending (all k < i-1)
    StageTerm beta[4];            // coef = beta (multiplied by the instance dt on device)
    double beta_cur;              // coefficient of L(u^(i-1)) (0 if unused)
    int store_deriv;              // derivative buffer to store L(u^(i-1)) into, or -1
    int last;                     // final stage: also computes the next CFL dt
};
struct IntegratorPlan {
    int n_stages;
    int n_state_bufs;             // state buffers (buffer 0 holds u^n at step start)
    int n_deriv_bufs;
    int result_buf;               // buffer holding u^{n+1} after the step
    StagePlan stage[4];
};
// Builds the plan; buffers are reused when a stage's output can overwrite a
// state that is only read pointwise from then on.  The current state rotates:
// a step starts from state buffer `start` and ends in plan.result_buf(start).
IntegratorPlan make_plan(int integrator);

// ---------------------------------------------------------------------------
// plain FP64 form (hc_plain.cu)
// ---------------------------------------------------------------------------

struct PlainParams {
    int dim;
    int gs[3];            // gridSize with ghosts
    int stepsize[3];
    long long numCells;
    double grid_dx[3];
    int bc[6];
    int fluxLimiter, recon, slopeLimiter;
    double gamma, rhoMin, PMin;
    int flux;             // HC_FLUX_*
    int hllcMethod;       // euler-hllc's hllcMethod, 0..2
    int entropyFix;       // Roe: useEntropyFluxFix, with its factor
    double entropyFactor;
    double fixedCons[6][5];   // HC_BOUNDARY_FIXED sides
};

struct PlainSolver;   // defined in hc_plain.cu
int plain_create(const hc_solver_desc& d, cudaStream_t stream, PlainSolver** out);
void plain_destroy(PlainSolver* p);
int plain_set_full(PlainSolver* p, const double* host_aos6);
int plain_get_full(PlainSolver* p, double* host_aos6);
int plain_set_interior(PlainSolver* p, const void* host, int layout);
int plain_get_interior(PlainSolver* p, void* host, int layout);
int plain_boundary(PlainSolver* p);
int plain_constrain_u(PlainSolver* p);
int plain_calc_dt(PlainSolver* p, double cfl, double fixed_dt, double* dt);
int plain_step(PlainSolver* p, int integrator, double dt);
int plain_conservation(PlainSolver* p, double sums[5]);
long long plain_num_cells(const PlainSolver* p);
const double* plain_state_dev(const PlainSolver* p);   // UBuf (AoS-6 FP64, ghosts included) on the device

// ---------------------------------------------------------------------------
// fused form (hc_fused.cu): a set of instances advanced together
// ---------------------------------------------------------------------------

struct FusedSet;      // defined in hc_fused.cu
struct FusedScheme {
    int precision;     // HC_F32_FUSED or HC_F64_FUSED
    int flux_limiter, recon, slope_limiter, integrator;
    int flux;          // HC_FLUX_*
    int hllc_method;   // HC_HLLC_*
};
int fused_create(const FusedScheme& sch, int max_slots, cudaStream_t stream, FusedSet** out);
void fused_destroy(FusedSet* f);
// bytes an instance of this shape holds on the device
size_t fused_instance_bytes(const FusedSet* f, const hc_solver_desc& d);
// stop_on_error: a non-finite state or dt ends the instance (batches); the
// single-solver form steps on like the reference and only records the status.
// The initial state comes from `host` (in `layout`), else from `init` (built
// on the device), else it stays zero until a set_state.
// sync = 0 leaves the uploads and launches queued (the caller synchronises
// before the host buffer is reused).
int fused_add(FusedSet* f, int slot, const hc_solver_desc& d, const void* host, int layout,
              double t_end, long long max_steps, int stop_on_error, const hc_init* init = nullptr, int sync = 1);
int fused_remove(FusedSet* f, int slot);
int fused_set_state(FusedSet* f, int slot, const void* host, int layout, int reset);
// resetState from a device-built initial condition
int fused_init_state(FusedSet* f, int slot, const hc_init& ic);
int plain_init_state(PlainSolver* p, const hc_init& ic, const hc_solver_desc& d);
int plain_expand_full(const hc_solver_desc& d, const void* interior_dev, int layout, double* full_dev, cudaStream_t s);
// the slot's interior state into device memory (layout as for host I/O)
int fused_get_state_dev(FusedSet* f, int slot, void* dev, int layout);

// hc_viz.cu: display variables and views over a solver's interior state,
// AoS-6 FP64 on the device, `stride` cells between neighbours per axis
struct VizState {
    const double* U;       // the first interior cell
    long long stride[3];
    hc_solver_desc d;
};
int viz_display(const VizState& st, int var, int zero_border, double* out_dev, cudaStream_t s);
int viz_range(const VizState& st, int var, double out[4], cudaStream_t s);
int viz_render(const VizState& st, const hc_render& r, unsigned char* out_dev, cudaStream_t s);
// initial conditions (hc_init.cu): the interior in AoS-6 FP64, x fastest, into device memory
int init_validate(const hc_init& ic, const hc_solver_desc& d);
int init_fill(const hc_init& ic, const hc_solver_desc& d, double* dst, cudaStream_t s);
// sync = 0 leaves the copy queued (the caller synchronises before reading)
int fused_get_state(FusedSet* f, int slot, void* host, int layout, int sync = 1);
// many admissions from host states / many fetches, queued in one pass (no wait)
int fused_add_many(FusedSet* f, int n, const int* slots, const hc_solver_desc* descs, const void* const* hosts,
                   int layout, const double* t_end, const long long* max_steps, int stop_on_error, int* n_done);
int fused_get_state_many(FusedSet* f, int n, const int* slots, void* const* hosts, int layout);
size_t fused_state_bytes(const FusedSet* f, int slot, int layout);
int fused_reserve_staging(FusedSet* f, size_t bytes);
// Runs `steps` updates of every live instance (device-side completion tests).
int fused_steps(FusedSet* f, int steps);
int fused_steps_timed(FusedSet* f, int steps, double* stage_ms, int n_stage_ms, double* total_ms);
// One update of the given slot's instance with an explicit dt (-1: CFL dt).
int fused_step_dt(FusedSet* f, int slot, double dt);
int fused_calc_dt(FusedSet* f, int slot, double* dt);
// one Runge-Kutta stage of a slot's update (the first sets the step's
// coefficients, the last completes the step; t is not advanced)
int fused_stage(FusedSet* f, int slot, double dt, int stage);
int fused_num_stages(const FusedSet* f);
// the two layers next to face (axis, side) of the buffer stage `stage` reads,
// as AoS-6 doubles on the host: dir 1 reads the interior layers, dir 0 writes the ghosts
int fused_slab(FusedSet* f, int slot, int stage, int axis, int side, int dir, double* host);
int fused_boundary(FusedSet* f, int slot);
int fused_constrain_u(FusedSet* f, int slot);
struct SlotInfo { double t; double dt; long long steps; int active; int done; int status; };
int fused_slot_info(FusedSet* f, std::vector<SlotInfo>& out);
int fused_set_time(FusedSet* f, int slot, double t);
int fused_set_limits(FusedSet* f, int slot, double t_end, long long max_steps);
int fused_variant(const FusedSet* f, int dim);
int fused_conservation(FusedSet* f, int slot, double sums[5]);
int fused_stats(FusedSet* f, hc_batch_stats* st);
int fused_autotune(FusedSet* f, const char* cache_path);
// fused_autotune that leaves slot `slot`'s solve as it was
int fused_autotune_keep(FusedSet* f, int slot, const char* cache_path);
int fused_set_schedule(FusedSet* f, int dim, int variant);
int fused_sync(FusedSet* f);

}  // namespace hc
