// hc_fused_host.cu -- host side of the fused form: a set of instances
// (slots) that advance together, each with its own grid, boundary, CFL dt and
// end time, sharing one scheme (reconstruction, limiters, integrator).
//
// Per step: k_begin (per-slot exit test and CFL dt, on the device), then one
// persistent launch of the stage kernel per Runge-Kutta stage and per grid
// dimension present, each walking a work list of (slot, tile) items.  The
// step is captured once into a CUDA graph and replayed; the work lists and
// the per-slot control blocks live in device memory, so the graph stays valid
// while instances come and go (it is re-captured only when a work-list
// buffer is reallocated or the set of dimensions changes).
#include "hc_internal.h"
#include "hc_fused.cuh"
#include "hc_pool.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

namespace hc {

using namespace fz;

namespace fz {

__global__ void k_begin(DevCtl* ctl, const DevInst* inst, int nslots, int begin, int rotates, BetaTable bt, int* work) {
    int const s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < kWorkCounters) work[s] = 0;   // the marching kernels' work counters of the step's stages
    if (s >= nslots) return;
    DevCtl& c = ctl[s];
    if (c.stepping) {
        c.t = c.t + c.dt;       // solverbase.lua:3168
        c.steps += 1;
        c.stepping = 0;
        c.par ^= 1;
        c.rot ^= rotates;
    }
    if (!begin) return;
    c.dtmin[c.par ^ 1] = kInfBits;
    if (!c.active) return;
    const DevInst& I = inst[s];
    if (c.status != 0 && I.stop_on_error) { c.active = 0; c.done = 1; return; }
    // app.lua:1590: the exit test precedes the update
    if (c.t >= I.t_end || c.steps >= I.max_steps) { c.active = 0; c.done = 1; return; }
    double const dt = I.fixed_dt > 0 ? I.fixed_dt : I.cfl * __longlong_as_double((long long)c.dtmin[c.par]);
    if (!(dt > 0) || !isfinite(dt)) {
        // the reference reports a bad dt and steps on with it (solverbase.lua:3017-3019)
        c.status |= DEV_NONFINITE;
        if (I.stop_on_error || !(dt == dt)) { c.active = 0; c.done = 1; return; }
    }
    c.dt = dt;
    fillStepCoefs(c, I, bt, dt);
    c.stepping = 1;
}

// Explicit-dt step of one slot (SolverBase:step(dt): t is not advanced).
__global__ void k_set_dt(DevCtl* ctl, const DevInst* inst, int slot, double dt, int on, int rotates, BetaTable bt,
                         int* work) {
    DevCtl& c = ctl[slot];
    for (int k = 0; k < kWorkCounters; ++k) work[k] = 0;
    if (on) {
        c.dtmin[c.par ^ 1] = kInfBits;
        c.dt = dt;
        fillStepCoefs(c, inst[slot], bt, dt);
        c.stepping = 1;
    } else {
        c.stepping = 0;
        c.par ^= 1;
        c.rot ^= rotates;
    }
}

__global__ void k_reset_dtmin(DevCtl* ctl, int slot) {
    ctl[slot].dtmin[ctl[slot].par] = kInfBits;
}

// A fresh state (resetState): clear time, step count and status; the dt
// parity and the buffer rotation stay, since they locate the state.
__global__ void k_restart(DevCtl* ctl, int slot) {
    DevCtl& c = ctl[slot];
    c.t = 0.;
    c.dt = 0.;
    c.steps = 0;
    c.status = 0;
    c.done = 0;
    c.active = 1;
    c.stepping = 0;
}

}  // namespace fz

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder() {
    if (g_encode) return HC_OK;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return fail(HC_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return HC_OK;
}

struct Registry {
    std::vector<StageLauncher> st;
    std::vector<AuxLauncher> aux;
    Registry() { register_launchers(st, aux); }
};
const Registry& registry() {
    static Registry r;
    return r;
}
const std::vector<StageLauncher>& stage_launchers() { return registry().st; }
const std::vector<AuxLauncher>& aux_launchers() { return registry().aux; }

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr int kMaxVariants = 32;   // schedule numbers the autotuner tries

}  // namespace

struct Slot {
    bool used = false;
    hc_solver_desc d;
    int dim = 0;
    size_t bytes = 0;
    void* mem = nullptr;
    DevInst inst;
    long long cells = 0;
};

struct FusedSet {
    FusedScheme sch;
    IntegratorPlan plan[1];        // stages from state buffer 0
    bool rotates = false;          // the plan leaves the state in plan.result_buf (per-slot DevCtl::rot)
    int rot_buf = 0;
    BetaTable betas;               // beta coefficients of the plan, for the per-step coefficients
    int esize = 4;
    int max_slots = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    std::vector<Slot> slots;
    DevInst* d_inst = nullptr;
    DevCtl* d_ctl = nullptr;
    CUtensorMap* d_tmaps = nullptr;
    // pinned host sources of the per-slot uploads (tensor maps, DevInst,
    // DevCtl), so that the copies are asynchronous; an entry is rewritten only
    // after the stream has drained the copy that last read it
    CUtensorMap* h_tmaps = nullptr;
    DevInst* h_inst_up = nullptr;
    DevCtl* h_ctl_up = nullptr;
    int* d_err = nullptr;
    int* d_work = nullptr;         // [kWorkCounters] work counters of the marching kernels
    int force_timeout = 0;         // test knob (HC_TEST_FORCE_TIMEOUT at creation): bounded waits count as run out
    DevCtl* h_ctl = nullptr;       // pinned mirror
    double* d_partial = nullptr;
    void* staging = nullptr;
    size_t staging_bytes = 0;
    // work lists per dimension
    int4* d_items[3] = {nullptr, nullptr, nullptr};
    size_t items_cap[3] = {0, 0, 0};
    int* d_nitems = nullptr;       // [6]: items per dimension, then the marching segment length per dimension
    int h_nitems[6] = {0, 0, 0, 0, 0, 0};
    bool items_dirty = true;
    // chosen tile-shape variant per dimension
    const StageLauncher* launcher[3] = {nullptr, nullptr, nullptr};
    int grid[3] = {0, 0, 0};
    int seg[3] = {0, 0, 0};        // marching launchers: rows (2D) / planes (3D) per segment of the item list
    int seg_fixed = 0;             // HC_MARCH_SEGMENT at creation: segments of min(this, the schedule's); 0 balanced
    // graph of one (or two, when the state rotates) steps
    cudaGraphExec_t graph = nullptr;
    // a branch per grid dimension inside the graph: the dimensions' stage
    // launches are independent, so an underfilled launch of one overlaps the
    // others (side streams and events used only while capturing)
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[3] = {nullptr, nullptr, nullptr};
    bool graph_valid = false;
    int extrap_dims = 0;           // dims (bit d-1) whose live instances have a linear / quadratic boundary
    int graph_dims_mask = 0;
    std::string tune_log;          // per-variant timings of the last autotune
    DevicePool pool;               // instance state buffers
};

static const StageLauncher* find_launcher(const FusedScheme& sch, int dim, int variant) {
    // the reconstruction a kernel must provide: 0 when the interface states
    // are the cells themselves (no PLM, or "piecewise constant")
    int const want = sch.recon >= HC_RECON_PLM_CONS ? sch.recon : 0;
    // only the Roe flux takes the flux limiter (fvsolver.lua:62-64)
    bool const lim = sch.flux_limiter > 0 && sch.flux == HC_FLUX_ROE;
    // prefer the reconstruction compiled in over any-kind (-1), then the
    // slope limiter compiled in over any (-1)
    const StageLauncher* best = nullptr;
    int bestScore = -1;
    for (const StageLauncher& L : stage_launchers()) {
        if (L.precision != sch.precision || L.dim != dim || L.lim != lim || L.variant != variant) continue;
        if (L.flux >= 0 && L.flux != sch.flux) continue;
        if (want == 0 ? L.recon != 0 : (L.recon != want && L.recon != -1)) continue;
        if (want != 0 && L.slope >= 0 && L.slope != sch.slope_limiter) continue;
        int const score = (L.recon == want ? 2 : 0) + (L.slope >= 0 ? 1 : 0);
        if (score > bestScore) {
            best = &L;
            bestScore = score;
        }
    }
    return best;
}

static const AuxLauncher* find_aux(int precision, int dim) {
    for (const AuxLauncher& A : aux_launchers())
        if (A.precision == precision && A.dim == dim) return &A;
    return nullptr;
}

static int set_launcher(FusedSet* f, int dim, int variant) {
    const StageLauncher* L = find_launcher(f->sch, dim, variant);
    if (!L) return fail(HC_ERR_INVALID, "no stage kernel for this scheme / dimension / variant");
    int const occ = L->occupancy();
    if (occ <= 0) return fail(HC_ERR_CUDA, "stage kernel cannot be resident (shared memory / registers)");
    f->launcher[dim - 1] = L;
    f->grid[dim - 1] = f->num_sms * occ;
    return HC_OK;
}

int fused_create(const FusedScheme& sch, int max_slots, cudaStream_t stream, FusedSet** out) {
    if (sch.precision != HC_F32_FUSED && sch.precision != HC_F64_FUSED) return fail(HC_ERR_INVALID, "fused precision");
    if (sch.recon != HC_RECON_NONE && sch.flux_limiter > 0)
        return fail(HC_ERR_INVALID, "usePLM together with a flux limiter (gridsolver.lua:119 asserts against it)");
    if (sch.integrator < 0 || sch.integrator >= HC_NUM_INTEGRATORS) return fail(HC_ERR_INVALID, "integrator");
    if (sch.flux_limiter < 0 || sch.flux_limiter >= HC_NUM_LIMITERS || sch.slope_limiter < 0 || sch.slope_limiter >= HC_NUM_LIMITERS)
        return fail(HC_ERR_INVALID, "limiter");
    if (max_slots <= 0) return fail(HC_ERR_INVALID, "max_slots");
    HC_CHECK(get_encoder());
    FusedSet* f = new FusedSet();
    f->sch = sch;
    {
        // test knob for the bounded-wait path; off unless the variable is "1"
        const char* ft = std::getenv("HC_TEST_FORCE_TIMEOUT");
        f->force_timeout = ft && ft[0] == '1' && ft[1] == 0;
        // tuning knob: a fixed marching segment length instead of the balanced one
        const char* sg = std::getenv("HC_MARCH_SEGMENT");
        f->seg_fixed = sg ? std::max(0, std::atoi(sg)) : 0;
    }
    f->esize = sch.precision == HC_F32_FUSED ? 4 : 8;
    f->max_slots = max_slots;
    f->stream = stream;
    f->plan[0] = make_plan(sch.integrator);
    f->rotates = f->plan[0].result_buf != 0;
    f->rot_buf = f->rotates ? f->plan[0].result_buf : 0;
    std::memset(&f->betas, 0, sizeof(f->betas));
    for (int st = 0; st < f->plan[0].n_stages; ++st) {
        const StagePlan& S = f->plan[0].stage[st];
        for (int m = 0; m < S.n_beta; ++m) f->betas.b[st][m] = S.beta[m].coef;
        f->betas.b[st][4] = S.beta_cur;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&f->num_sms, cudaDevAttrMultiProcessorCount, dev);
    f->slots.resize(max_slots);
    int r = HC_OK;
    auto A = [&](void** p, size_t b) {
        if (r != HC_OK) return;
        cudaError_t e = cudaMalloc(p, b);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMalloc");
    };
    A((void**)&f->d_inst, sizeof(DevInst) * max_slots);
    A((void**)&f->d_ctl, sizeof(DevCtl) * max_slots);
    A((void**)&f->d_tmaps, sizeof(CUtensorMap) * kMaxBufs * max_slots);
    A((void**)&f->d_err, sizeof(int));
    A((void**)&f->d_work, sizeof(int) * kWorkCounters);
    A((void**)&f->d_nitems, sizeof(int) * 6);
    A((void**)&f->d_partial, sizeof(double) * 5 * 1024);
    auto H = [&](void** p, size_t b) {
        if (r != HC_OK) return;
        cudaError_t e = cudaMallocHost(p, b);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMallocHost");
        else std::memset(*p, 0, b);
    };
    H((void**)&f->h_ctl, sizeof(DevCtl) * max_slots);
    H((void**)&f->h_tmaps, sizeof(CUtensorMap) * kMaxBufs * max_slots);
    H((void**)&f->h_inst_up, sizeof(DevInst) * max_slots);
    H((void**)&f->h_ctl_up, sizeof(DevCtl) * max_slots);
    if (r == HC_OK) {
        cudaMemsetAsync(f->d_inst, 0, sizeof(DevInst) * max_slots, stream);
        cudaMemsetAsync(f->d_ctl, 0, sizeof(DevCtl) * max_slots, stream);
        cudaMemsetAsync(f->d_tmaps, 0, sizeof(CUtensorMap) * kMaxBufs * max_slots, stream);
        cudaMemsetAsync(f->d_err, 0, sizeof(int), stream);
        cudaMemsetAsync(f->d_work, 0, sizeof(int) * kWorkCounters, stream);
        cudaMemsetAsync(f->d_nitems, 0, sizeof(int) * 6, stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemsetAsync");
    }
    for (int dim = 1; dim <= 3 && r == HC_OK; ++dim) r = set_launcher(f, dim, 0);
    if (r != HC_OK) {
        fused_destroy(f);
        return r;
    }
    *out = f;
    return HC_OK;
}

void fused_destroy(FusedSet* f) {
    if (!f) return;
    if (f->stream) cudaStreamSynchronize(f->stream);
    f->pool.release_all();
    cudaFree(f->d_inst);
    cudaFree(f->d_ctl);
    cudaFree(f->d_tmaps);
    cudaFree(f->d_err);
    cudaFree(f->d_work);
    cudaFree(f->d_nitems);
    cudaFree(f->d_partial);
    cudaFree(f->staging);
    for (int d = 0; d < 3; ++d) cudaFree(f->d_items[d]);
    if (f->h_ctl) cudaFreeHost(f->h_ctl);
    if (f->h_tmaps) cudaFreeHost(f->h_tmaps);
    if (f->h_inst_up) cudaFreeHost(f->h_inst_up);
    if (f->h_ctl_up) cudaFreeHost(f->h_ctl_up);
    if (f->graph) cudaGraphExecDestroy(f->graph);
    for (int d = 0; d < 3; ++d) {
        if (f->side[d]) cudaStreamDestroy(f->side[d]);
        if (f->join[d]) cudaEventDestroy(f->join[d]);
    }
    if (f->fork) cudaEventDestroy(f->fork);
    delete f;
}

static void padded_dims(const hc_solver_desc& d, int& px, int& py, int& pz) {
    px = (int)round_up((size_t)d.n[0] + 2 * kG, 32);
    py = d.dim > 1 ? d.n[1] + 2 * kG : 1;
    pz = d.dim > 2 ? d.n[2] + 2 * kG : 1;
}

size_t fused_instance_bytes(const FusedSet* f, const hc_solver_desc& d) {
    int px, py, pz;
    padded_dims(d, px, py, pz);
    size_t const planeBytes = round_up((size_t)px * py * pz * f->esize, 256);
    return planeBytes * 5 * (size_t)(f->plan[0].n_state_bufs + f->plan[0].n_deriv_bufs);
}

static int validate(const FusedSet* f, const hc_solver_desc& d) {
    if (d.dim < 1 || d.dim > 3) return fail(HC_ERR_INVALID, "dim must be 1, 2 or 3");
    for (int k = 0; k < d.dim; ++k) {
        if (d.n[k] < 2) return fail(HC_ERR_INVALID, "each active axis needs at least 2 cells");
        if (d.n[k] > (1 << 24)) return fail(HC_ERR_INVALID, "grid axis too large");
        if (!(d.maxs[k] > d.mins[k])) return fail(HC_ERR_INVALID, "maxs must exceed mins");
    }
    // 'none' leaves a side's ghost cells as they are (gridsolver.lua's
    // BoundaryNone): a caller fills them, as a grid cut into slabs does with
    // its neighbours' layers
    for (int k = 0; k < 2 * d.dim; ++k)
        if (d.boundary[k] < 0 || d.boundary[k] >= HC_NUM_BOUNDARIES)
            return fail(HC_ERR_INVALID, "the fused form supports none, periodic, mirror, freeflow, linear and quadratic boundaries");
    for (int k = 0; k < d.dim; ++k)
        if ((d.boundary[2 * k] == HC_BOUNDARY_PERIODIC) != (d.boundary[2 * k + 1] == HC_BOUNDARY_PERIODIC))
            return fail(HC_ERR_INVALID, "periodic boundaries must be periodic on both sides of an axis");
    if (!(d.gamma > 1.)) return fail(HC_ERR_INVALID, "gamma must exceed 1");
    (void)f;
    return HC_OK;
}

// Tensor maps of a slot's state buffers for the launcher's box (into the
// pinned mirror; with `upload`, also to the device).
static int encode_maps(FusedSet* f, int slot, bool upload = true) {
    Slot& S = f->slots[slot];
    const StageLauncher* L = f->launcher[S.dim - 1];
    const DevInst& I = S.inst;
    CUtensorMapDataType const dt = f->esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    int const rank = S.dim + 1;
    cuuint64_t gdim[5], gstride[4];
    cuuint32_t box[5], estride[5] = {1, 1, 1, 1, 1};
    size_t const es = f->esize;
    gdim[0] = I.px;
    box[0] = L->box[0];
    if (S.dim == 1) {
        gdim[1] = 5; box[1] = 5;
        gstride[0] = I.plane * es;
    } else if (S.dim == 2) {
        gdim[1] = I.py; gdim[2] = 5;
        box[1] = L->box[1]; box[2] = 5;
        gstride[0] = (cuuint64_t)I.px * es;
        gstride[1] = I.plane * es;
    } else {
        gdim[1] = I.py; gdim[2] = I.pz; gdim[3] = 5;
        box[1] = L->box[1]; box[2] = L->box[2]; box[3] = 5;
        gstride[0] = (cuuint64_t)I.px * es;
        gstride[1] = (cuuint64_t)I.px * I.py * es;
        gstride[2] = I.plane * es;
    }
    for (int b = 0; b < f->plan[0].n_state_bufs; ++b) {
        CUtensorMap* m = &f->h_tmaps[(size_t)slot * kMaxBufs + b];
        CUresult r = g_encode(m, dt, rank, I.buf[b], gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(HC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    if (upload)
        HC_CUDA(cudaMemcpyAsync(f->d_tmaps + (size_t)slot * kMaxBufs, &f->h_tmaps[(size_t)slot * kMaxBufs],
                                sizeof(CUtensorMap) * kMaxBufs, cudaMemcpyHostToDevice, f->stream));
    return HC_OK;
}

static int ensure_staging(FusedSet* f, size_t bytes) {
    if (f->staging_bytes >= bytes) return HC_OK;
    HC_CUDA(cudaStreamSynchronize(f->stream));
    cudaFree(f->staging);
    f->staging = nullptr;
    f->staging_bytes = 0;
    size_t const cap = std::max(bytes, (size_t)1 << 20);
    HC_CUDA(cudaMalloc(&f->staging, cap));
    f->staging_bytes = cap;
    return HC_OK;
}

static size_t layout_bytes(long long n, int layout) {
    return layout == HC_LAYOUT_AOS6_F64 ? n * 6 * sizeof(double)
         : layout == HC_LAYOUT_SOA5_F64 ? n * 5 * sizeof(double) : n * 5 * sizeof(float);
}

// the instance has a linear or quadratic side (ghosts from neighbours)
static bool has_extrap(const Slot& S) {
    for (int k = 0; k < 2 * S.dim; ++k)
        if (S.inst.bc[k] == HC_BOUNDARY_LINEAR || S.inst.bc[k] == HC_BOUNDARY_QUADRATIC) return true;
    return false;
}

// the instance has a fixed side (constant ghosts, set once)
static bool has_fixed(const Slot& S) {
    for (int k = 0; k < 2 * S.dim; ++k)
        if (S.inst.bc[k] == HC_BOUNDARY_FIXED) return true;
    return false;
}

// buffer holding a slot's current state
static int state_buf(FusedSet* f, int slot) {
    if (!f->rotates) return 0;
    int rot = 0;
    cudaMemcpyAsync(&rot, &f->d_ctl[slot].rot, sizeof(int), cudaMemcpyDeviceToHost, f->stream);
    cudaStreamSynchronize(f->stream);
    return rot ? f->rot_buf : 0;
}

// fresh: the slot's DevCtl was just uploaded in its reset form (time, steps,
// status zero, active, both dt minima +inf, parity 0, no buffer rotation), so
// the two control kernels that would write the same values are not launched
// and the state goes to buffer 0.
static int set_state(FusedSet* f, int slot, const void* host, int layout, int reset, bool fresh) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    size_t const bytes = layout_bytes(S.cells, layout);
    HC_CHECK(ensure_staging(f, bytes));
    HC_CUDA(cudaMemcpyAsync(f->staging, host, bytes, cudaMemcpyHostToDevice, f->stream));
    int const b = fresh ? 0 : state_buf(f, slot);
    if (reset && !fresh) fz::k_restart<<<1, 1, 0, f->stream>>>(f->d_ctl, slot);
    if (!fresh) fz::k_reset_dtmin<<<1, 1, 0, f->stream>>>(f->d_ctl, slot);
    A->load(f->d_inst, f->d_ctl, slot, b, f->staging, layout, reset, S.cells, f->stream);
    if (has_extrap(S)) A->extrap_slot(f->d_inst, slot, b, f->stream);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_set_state(FusedSet* f, int slot, const void* host, int layout, int reset) {
    return set_state(f, slot, host, layout, reset, false);
}

static int init_state(FusedSet* f, int slot, const hc_init& ic, bool fresh) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    HC_CHECK(init_validate(ic, S.d));
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    HC_CHECK(ensure_staging(f, layout_bytes(S.cells, HC_LAYOUT_AOS6_F64)));
    HC_CHECK(init_fill(ic, S.d, static_cast<double*>(f->staging), f->stream));
    // from here on exactly the path of a host upload (fused_set_state with reset)
    int const b = fresh ? 0 : state_buf(f, slot);
    if (!fresh) fz::k_restart<<<1, 1, 0, f->stream>>>(f->d_ctl, slot);
    if (!fresh) fz::k_reset_dtmin<<<1, 1, 0, f->stream>>>(f->d_ctl, slot);
    A->load(f->d_inst, f->d_ctl, slot, b, f->staging, HC_LAYOUT_AOS6_F64, 1, S.cells, f->stream);
    if (has_extrap(S)) A->extrap_slot(f->d_inst, slot, b, f->stream);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_init_state(FusedSet* f, int slot, const hc_init& ic) { return init_state(f, slot, ic, false); }

int fused_get_state_dev(FusedSet* f, int slot, void* dev, int layout) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    find_aux(f->sch.precision, S.dim)->xfer(f->d_inst, slot, state_buf(f, slot), dev, layout, 1, S.cells, f->stream);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_get_state(FusedSet* f, int slot, void* host, int layout, int sync) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    size_t const bytes = layout_bytes(S.cells, layout);
    // one staging buffer serves every queued fetch: each gather waits in
    // stream order for the previous copy out of it
    HC_CHECK(ensure_staging(f, bytes));
    A->xfer(f->d_inst, slot, state_buf(f, slot), f->staging, layout, 1, S.cells, f->stream);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaMemcpyAsync(host, f->staging, bytes, cudaMemcpyDeviceToHost, f->stream));
    if (sync) HC_CUDA(cudaStreamSynchronize(f->stream));
    return HC_OK;
}

size_t fused_state_bytes(const FusedSet* f, int slot, int layout) {
    return layout_bytes(f->slots[slot].cells, layout);
}

int fused_reserve_staging(FusedSet* f, size_t bytes) { return ensure_staging(f, bytes); }

// The host side of an admission: the slot's device memory (zeroed on the
// stream), its descriptor and control block in the pinned mirrors and its
// tensor maps; uploading them is the caller's (upload_slots).
static int add_host(FusedSet* f, int slot, const hc_solver_desc& d, double t_end, long long max_steps,
                    int stop_on_error, bool zero = true) {
    if (slot < 0 || slot >= f->max_slots || f->slots[slot].used) return fail(HC_ERR_STATE, "slot unavailable");
    HC_CHECK(validate(f, d));
    Slot& S = f->slots[slot];
    S.d = d;
    S.dim = d.dim;
    int px, py, pz;
    padded_dims(d, px, py, pz);
    size_t const plane = (size_t)px * py * pz;
    size_t const planeBytes = round_up(plane * f->esize, 256);
    int const nb = f->plan[0].n_state_bufs, nd = f->plan[0].n_deriv_bufs;
    S.bytes = planeBytes * 5 * (nb + nd);
    cudaError_t e = f->pool.alloc(S.bytes, &S.mem);
    if (e != cudaSuccess) { S.mem = nullptr; return cuda_fail(e, "cudaMalloc (instance state)"); }
    if (zero) HC_CUDA(cudaMemsetAsync(S.mem, 0, S.bytes, f->stream));
    DevInst& I = S.inst;
    std::memset(&I, 0, sizeof(I));
    I.dim = d.dim;
    for (int k = 0; k < 3; ++k) I.n[k] = k < d.dim ? d.n[k] : 1;
    S.cells = (long long)I.n[0] * I.n[1] * I.n[2];
    I.px = px; I.py = py; I.pz = pz;
    I.plane = (long long)(planeBytes / f->esize);
    for (int k = 0; k < 6; ++k) I.bc[k] = d.boundary[k];
    // grid_dx and the calcDerivFromFlux / calcFlux area factors, evaluated in
    // double in the reference's order (fvsolver.cl:37-102, fvsolver.lua:97-111)
    for (int k = 0; k < 3; ++k) I.grid_dx[k] = (d.maxs[k] - d.mins[k]) / (double)(k < d.dim ? d.n[k] : 1);
    double volume = 1.;
    for (int k = 0; k < d.dim; ++k) volume = volume * I.grid_dx[k];
    for (int side = 0; side < 3; ++side) {
        double area = 1.;
        for (int k = 0; k < d.dim; ++k) if (k != side) area = area * I.grid_dx[k];
        I.zeroFlux[side] = area <= 1e-7;
        if (volume > 1e-7) {
            double const invVolume = 1. / volume;
            double a = area;
            if (a <= 1e-7) a = 0.;
            a *= invVolume;
            I.area[side] = a;
            I.skipDeriv[side] = 0;
        } else {
            I.area[side] = 0.;
            I.skipDeriv[side] = 1;
        }
    }
    I.gamma = d.gamma;
    I.rhoMin = d.rho_min;
    I.PMin = d.p_min;
    I.cfl = d.cfl;
    I.fixed_dt = d.fixed_dt;
    I.t_end = t_end;
    I.max_steps = max_steps;
    I.stop_on_error = stop_on_error;
    I.f_gamma = (float)d.gamma;
    I.f_g1 = (float)(d.gamma - 1.);
    I.f_rhoMin = (float)d.rho_min;
    I.f_PMin = (float)d.p_min;
    I.f_invg1 = (float)(1. / (d.gamma - 1.));
    I.entropyFix = d.entropy_fix != 0;
    I.entropyFactor = d.entropy_fix_factor;
    I.f_entropyFactor = d.entropy_fix ? (float)d.entropy_fix_factor : 0.f;
    std::memcpy(I.fixedCons, d.fixed_cons, sizeof(I.fixedCons));
    for (int k = 0; k < 3; ++k) {
        I.f_area[k] = (float)I.area[k];
        I.f_gdx[k] = (float)I.grid_dx[k];
    }
    char* p = (char*)S.mem;
    for (int b = 0; b < nb; ++b, p += planeBytes * 5) I.buf[b] = p;
    for (int b = 0; b < nd; ++b, p += planeBytes * 5) I.dbuf[b] = p;
    S.used = true;
    f->h_inst_up[slot] = I;
    DevCtl& c = f->h_ctl_up[slot];
    std::memset(&c, 0, sizeof(c));
    c.dtmin[0] = c.dtmin[1] = kInfBits;
    c.active = 1;
    int const r = encode_maps(f, slot, false);
    if (r != HC_OK) fused_remove(f, slot);
    return r;
}

// Descriptors, control blocks and tensor maps of slots [lo, hi) from the
// pinned mirrors, one copy each.
static int upload_slots(FusedSet* f, int lo, int hi) {
    size_t const n = (size_t)(hi - lo);
    HC_CUDA(cudaMemcpyAsync(f->d_inst + lo, &f->h_inst_up[lo], sizeof(DevInst) * n, cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaMemcpyAsync(f->d_ctl + lo, &f->h_ctl_up[lo], sizeof(DevCtl) * n, cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaMemcpyAsync(f->d_tmaps + (size_t)lo * kMaxBufs, &f->h_tmaps[(size_t)lo * kMaxBufs],
                            sizeof(CUtensorMap) * kMaxBufs * n, cudaMemcpyHostToDevice, f->stream));
    return HC_OK;
}

int fused_add(FusedSet* f, int slot, const hc_solver_desc& d, const void* host, int layout, double t_end, long long max_steps,
              int stop_on_error, const hc_init* init, int sync) {
    HC_CHECK(add_host(f, slot, d, t_end, max_steps, stop_on_error));
    Slot& S = f->slots[slot];
    int r = upload_slots(f, slot, slot + 1);
    if (r == HC_OK && has_fixed(S))
        find_aux(f->sch.precision, S.dim)->fixed_ghosts(f->d_inst, slot, f->plan[0].n_state_bufs, f->stream);
    if (r == HC_OK && host) r = set_state(f, slot, host, layout, 1, true);
    if (r == HC_OK && !host && init) r = init_state(f, slot, *init, true);
    if (r != HC_OK) {
        fused_remove(f, slot);
        return r;
    }
    f->items_dirty = true;
    if (sync) HC_CUDA(cudaStreamSynchronize(f->stream));
    return HC_OK;
}

// The device address of a host buffer in page-locked memory (cudaMallocHost,
// cudaHostRegister), which kernels read and write in place over the host link;
// nullptr for pageable memory.
static void* pinned_device_ptr(const void* host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Batched set-up (load) or gather passes over n instances: one launch per
// grid dimension and kXferJobs instances; job j moves state buffer bufs[j] of
// slots[j] from / to hosts[j].
static void run_jobs(FusedSet* f, int n, const int* slots, const int* bufs, void* const* hosts, int layout, bool load) {
    for (int dim = 1; dim <= 3; ++dim) {
        const AuxLauncher* A = find_aux(f->sch.precision, dim);
        fz::XferJobs J;
        J.n = 0;
        J.first[0] = 0;
        auto flush = [&]() {
            if (!J.n) return;
            if (load) A->load_many(f->d_inst, f->d_ctl, J, layout, 1, f->stream);
            else A->xfer_many(f->d_inst, J, layout, 1, f->stream);
            J.n = 0;
        };
        for (int j = 0; j < n; ++j) {
            const Slot& S = f->slots[slots[j]];
            if (S.dim != dim) continue;
            J.slot[J.n] = slots[j];
            J.buf[J.n] = bufs[j];
            J.host[J.n] = hosts[j];
            J.first[J.n + 1] = J.first[J.n] + (int)((S.cells + fz::kJobCells - 1) / fz::kJobCells);
            if (++J.n == fz::kXferJobs) flush();
        }
        flush();
    }
}

// The device side of admitting `done` instances whose host side add_host has
// set up (zeroing not yet done): memory zeroed, descriptors uploaded, state
// set up from hosts[j].
static int setup_many(FusedSet* f, int done, const int* slots, const void* const* hosts, int layout) {
    {
        // the instances' memory zeroed: one memset per run of adjacent pool ranges
        std::vector<std::pair<char*, size_t>> ranges(done);
        for (int j = 0; j < done; ++j) ranges[j] = {(char*)f->slots[slots[j]].mem, f->slots[slots[j]].bytes};
        std::sort(ranges.begin(), ranges.end());
        for (size_t a = 0; a < ranges.size();) {
            char* const lo = ranges[a].first;
            char* hi = lo + ranges[a].second;
            size_t b = a + 1;
            while (b < ranges.size() && ranges[b].first == hi) hi += ranges[b++].second;
            HC_CUDA(cudaMemsetAsync(lo, 0, (size_t)(hi - lo), f->stream));
            a = b;
        }
    }
    std::vector<int> sorted(slots, slots + done);
    std::sort(sorted.begin(), sorted.end());
    for (size_t a = 0; a < sorted.size();) {
        size_t b = a + 1;
        while (b < sorted.size() && sorted[b] == sorted[b - 1] + 1) ++b;
        HC_CHECK(upload_slots(f, sorted[a], sorted[b - 1] + 1));
        a = b;
    }
    std::vector<void*> direct(done);
    std::vector<size_t> off(done + 1, 0);
    for (int j = 0; j < done; ++j) {
        direct[j] = pinned_device_ptr(hosts[j]);
        off[j + 1] = off[j] + (direct[j] ? 0 : round_up(layout_bytes(f->slots[slots[j]].cells, layout), 256));
    }
    if (off[done]) HC_CHECK(ensure_staging(f, off[done]));
    // fixed ghosts first, then the set-up passes, then the linear / quadratic
    // ghosts (which read the interior)
    std::vector<void*> src(done);
    for (int j = 0; j < done; ++j) {
        Slot& S = f->slots[slots[j]];
        if (has_fixed(S)) find_aux(f->sch.precision, S.dim)->fixed_ghosts(f->d_inst, slots[j], f->plan[0].n_state_bufs,
                                                                         f->stream);
        src[j] = direct[j];
        if (!src[j]) {
            src[j] = static_cast<char*>(f->staging) + off[j];
            HC_CUDA(cudaMemcpyAsync(src[j], hosts[j], layout_bytes(S.cells, layout), cudaMemcpyHostToDevice, f->stream));
        }
    }
    std::vector<int> bufs(done, 0);
    run_jobs(f, done, slots, bufs.data(), src.data(), layout, true);
    for (int j = 0; j < done; ++j) {
        Slot& S = f->slots[slots[j]];
        if (has_extrap(S)) find_aux(f->sch.precision, S.dim)->extrap_slot(f->d_inst, slots[j], 0, f->stream);
    }
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

// n admissions from host states, in chunks of one set-up launch's instances:
// the host side of each, then the chunk's memory zeroed, its descriptors
// uploaded in runs of consecutive slots and its states set up by batched
// load launches (a page-locked host buffer read in place, any other through
// its own range of one staging buffer), all queued back to back (no wait).
// Stops at the first instance the host side refuses; *n_done = the instances
// admitted.
int fused_add_many(FusedSet* f, int n, const int* slots, const hc_solver_desc* descs, const void* const* hosts,
                   int layout, const double* t_end, const long long* max_steps, int stop_on_error, int* n_done) {
    *n_done = 0;
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    int r = HC_OK;
    int k = 0;
    // in chunks of one set-up launch's instances: the device sets up a chunk
    // while the host prepares the next
    while (k < n && r == HC_OK) {
        int const k0 = k, end = std::min(n, k0 + fz::kXferJobs);
        for (; k < end; ++k) {
            r = add_host(f, slots[k], descs[k], t_end[k], max_steps[k], stop_on_error, false);
            if (r != HC_OK) break;
        }
        *n_done = k;
        if (k > k0) {
            f->items_dirty = true;
            HC_CHECK(setup_many(f, k - k0, slots + k0, hosts + k0, layout));
        }
    }
    return r;
}

// n fetches in one pass: the slots' states gathered by batched launches (one
// per grid dimension and kXferJobs slots), straight into a page-locked host
// buffer, otherwise into the slot's own range of one staging buffer and
// copied out from there (the copies back to back); no wait.
int fused_get_state_many(FusedSet* f, int n, const int* slots, void* const* hosts, int layout) {
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    std::vector<void*> direct(n);
    std::vector<size_t> off(n + 1, 0);
    for (int j = 0; j < n; ++j) {
        const Slot& S = f->slots[slots[j]];
        if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
        direct[j] = pinned_device_ptr(hosts[j]);
        off[j + 1] = off[j] + (direct[j] ? 0 : round_up(layout_bytes(S.cells, layout), 256));
    }
    if (off[n]) HC_CHECK(ensure_staging(f, off[n]));
    std::vector<void*> dst(n);
    std::vector<int> bufs(n);
    for (int j = 0; j < n; ++j) {
        dst[j] = direct[j] ? direct[j] : static_cast<char*>(f->staging) + off[j];
        bufs[j] = state_buf(f, slots[j]);
    }
    run_jobs(f, n, slots, bufs.data(), dst.data(), layout, false);
    HC_CUDA(cudaGetLastError());
    for (int j = 0; j < n; ++j)
        if (!direct[j])
            HC_CUDA(cudaMemcpyAsync(hosts[j], static_cast<char*>(f->staging) + off[j],
                                    layout_bytes(f->slots[slots[j]].cells, layout), cudaMemcpyDeviceToHost, f->stream));
    return HC_OK;
}

int fused_remove(FusedSet* f, int slot) {
    if (slot < 0 || slot >= f->max_slots) return fail(HC_ERR_INVALID, "slot");
    Slot& S = f->slots[slot];
    if (!S.used) return HC_OK;
    // no synchronisation: later users of the range are ordered behind the
    // work already on the stream
    f->pool.release(S.mem, S.bytes);
    S.mem = nullptr;
    S.used = false;
    HC_CUDA(cudaMemsetAsync(f->d_ctl + slot, 0, sizeof(DevCtl), f->stream));
    f->items_dirty = true;
    return HC_OK;
}

// Segment length of a marching launcher's items over the active instances of
// dimension d + 1 (h_ctl current).  The schedule's own length, unless its
// items would fill fewer than two rounds of the launch's resident warps (2D:
// a warp per item) or CTAs (3D): then the length among 4 .. the schedule's
// that minimises rounds x (length + 4), the 4 rows or planes beside each
// segment that its box also loads, so one small grid still spreads over
// every SM.  The bits do not depend on it.
static int march_segment(const FusedSet* f, int d) {
    const StageLauncher* L = f->launcher[d];
    int const full = L->seg;
    if (f->seg_fixed > 0) return std::min(f->seg_fixed, full);
    long long const units = (long long)f->grid[d] * (d == 1 ? L->nthreads / 32 : 1);
    // per live instance: its strips (times its y tiles in 3D) and its extent
    // along the marching axis
    std::vector<std::pair<long long, int>> live;
    for (int s = 0; s < f->max_slots; ++s) {
        const Slot& S = f->slots[s];
        if (!S.used || !f->h_ctl[s].active || S.dim != d + 1) continue;
        long long const strips = (S.inst.n[0] + L->tx - 1) / L->tx;
        long long const tiles = d == 2 ? (S.inst.n[1] + L->ty - 1) / L->ty : 1;
        live.emplace_back(strips * tiles, S.inst.n[d]);
    }
    auto count = [&](int h) {
        long long n = 0;
        for (const auto& v : live) n += v.first * ((v.second + h - 1) / h);
        return n;
    };
    long long const nfull = count(full);
    if (nfull == 0 || nfull >= 2 * units) return full;
    int best = full;
    long long bestCost = (long long)((nfull + units - 1) / units) * (full + 4);
    for (int h = full - 1; h >= 4; --h) {
        long long const cost = (long long)((count(h) + units - 1) / units) * (h + 4);
        if (cost < bestCost) {
            best = h;
            bestCost = cost;
        }
    }
    return best;
}

// Rebuilds the per-dimension (slot, tile) work lists.  Items are ordered by
// slot, then z, y, x tile, so consecutive CTAs work on neighbouring tiles and
// share halo rows in L2.
static int rebuild_items(FusedSet* f) {
    if (!f->items_dirty) return HC_OK;
    HC_CUDA(cudaStreamSynchronize(f->stream));
    HC_CUDA(cudaMemcpy(f->h_ctl, f->d_ctl, sizeof(DevCtl) * f->max_slots, cudaMemcpyDeviceToHost));
    // read by the marching kernels from device memory, as the item counts
    // are, so a captured step graph stays valid when they change
    for (int d = 0; d < 3; ++d) {
        const StageLauncher* L = f->launcher[d];
        f->seg[d] = L && L->march ? march_segment(f, d) : 0;
    }
    std::vector<int4> items[3];
    int extrap = 0;
    for (int s = 0; s < f->max_slots; ++s) {
        const Slot& S = f->slots[s];
        if (!S.used || !f->h_ctl[s].active) continue;
        for (int k = 0; k < 2 * S.dim; ++k)
            if (S.inst.bc[k] == HC_BOUNDARY_LINEAR || S.inst.bc[k] == HC_BOUNDARY_QUADRATIC) extrap |= 1 << (S.dim - 1);
        const StageLauncher* L = f->launcher[S.dim - 1];
        // a marching launcher's segments run along y (2D) or z (3D)
        int const ty = L->march && S.dim == 2 ? f->seg[1] : L->ty;
        int const tz = L->march && S.dim == 3 ? f->seg[2] : L->tz;
        int const ntx = (S.inst.n[0] + L->tx - 1) / L->tx;
        int const nty = S.dim > 1 ? (S.inst.n[1] + ty - 1) / ty : 1;
        int const ntz = S.dim > 2 ? (S.inst.n[2] + tz - 1) / tz : 1;
        for (int z = 0; z < ntz; ++z)
            for (int y = 0; y < nty; ++y)
                for (int x = 0; x < ntx; ++x) items[S.dim - 1].push_back(make_int4(s, x, y, z));
    }
    // a marching schedule's item costs its segment's rows (times its planes
    // in 3D): full segments first, the shorter ones at the grid tops last, so
    // the launch's tail is short (stable: neighbouring strips stay together
    // for their halo rows in L2)
    for (int d = 0; d < 3; ++d) {
        const StageLauncher* L = f->launcher[d];
        if (!L || !L->march) continue;
        int const h = f->seg[d];
        auto rowsOf = [&](const int4& it) {
            const DevInst& I = f->slots[it.x].inst;
            if (d == 1) return std::min(h, I.n[1] - it.z * h);
            return std::min(L->ty, I.n[1] - it.z * L->ty) * std::min(h, I.n[2] - it.w * h);
        };
        std::stable_sort(items[d].begin(), items[d].end(),
                         [&](const int4& a, const int4& b) { return rowsOf(a) > rowsOf(b); });
    }
    int mask = 0;
    for (int d = 0; d < 3; ++d) {
        size_t const n = items[d].size();
        if (n) mask |= 1 << d;
        if (n > f->items_cap[d]) {
            cudaFree(f->d_items[d]);
            f->d_items[d] = nullptr;
            size_t const cap = std::max(n * 2, (size_t)1024);
            HC_CUDA(cudaMalloc(&f->d_items[d], cap * sizeof(int4)));
            f->items_cap[d] = cap;
            f->graph_valid = false;
        }
        if (n) HC_CUDA(cudaMemcpyAsync(f->d_items[d], items[d].data(), n * sizeof(int4), cudaMemcpyHostToDevice, f->stream));
        f->h_nitems[d] = (int)n;
    }
    for (int d = 0; d < 3; ++d) f->h_nitems[3 + d] = f->seg[d];
    HC_CUDA(cudaMemcpyAsync(f->d_nitems, f->h_nitems, sizeof(int) * 6, cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    if (mask != f->graph_dims_mask || extrap != f->extrap_dims) f->graph_valid = false;
    f->graph_dims_mask = mask;
    f->extrap_dims = extrap;
    f->items_dirty = false;
    return HC_OK;
}

static void fill_stage(StageDev& sd, const StagePlan& sp, int stage) {
    std::memset(&sd, 0, sizeof(sd));
    sd.stage = stage;
    sd.in_buf = sp.in_buf;
    sd.out_buf = sp.out_buf;
    sd.n_alpha = sp.n_alpha;
    for (int k = 0; k < sp.n_alpha; ++k) {
        sd.alpha_buf[k] = sp.alpha[k].buf;
        sd.alpha[k] = sp.alpha[k].coef;
        sd.alpha_f[k] = (float)sp.alpha[k].coef;
    }
    sd.n_beta = sp.n_beta;
    for (int k = 0; k < sp.n_beta; ++k) { sd.beta_buf[k] = sp.beta[k].buf; sd.beta[k] = sp.beta[k].coef; }
    sd.beta_cur = sp.beta_cur;
    sd.store_deriv = sp.store_deriv;
    sd.last = sp.last;
}

// Launches the stages of one step with plan p (k_begin / k_set_dt around it
// are the caller's).
static int launch_stages(FusedSet* f, const IntegratorPlan& P, int dims_mask, cudaStream_t stream = nullptr) {
    if (!stream) stream = f->stream;
    for (int s = 0; s < P.n_stages; ++s) {
        for (int d = 0; d < 3; ++d) {
            if (!(dims_mask & (1 << d))) continue;
            StageArgs a;
            a.inst = f->d_inst;
            a.ctl = f->d_ctl;
            a.tmaps = f->d_tmaps;
            a.items = f->d_items[d];
            a.nitems = f->d_nitems + d;
            a.seg = f->d_nitems + 3 + d;
            a.err = f->d_err;
            a.rot_buf = f->rot_buf;
            a.flux = f->sch.flux;
            a.hllcMethod = f->sch.hllc_method == HC_HLLC_DEFAULT ? 2 : f->sch.hllc_method - 1;
            a.recon = f->sch.recon;
            a.work = f->d_work + P.stage[s].index * 3 + d;
            a.force_timeout = f->force_timeout;
            fill_stage(a.st, P.stage[s], P.stage[s].index);
            f->launcher[d]->launch(a, f->sch.slope_limiter, f->sch.flux_limiter, f->grid[d], stream);
        }
        // linear / quadratic ghosts of this stage's output, before the next stage reads them
        for (int d = 0; d < 3; ++d)
            if ((dims_mask & f->extrap_dims) & (1 << d))
                find_aux(f->sch.precision, d + 1)->extrap_stage(f->d_inst, f->d_ctl, f->max_slots, P.stage[s].out_buf,
                                                                f->rot_buf, stream);
    }
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

static int launch_step(FusedSet* f, int dims_mask) {
    unsigned const g = (unsigned)((f->max_slots + 127) / 128);
    fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 1, f->rotates, f->betas, f->d_work);
    return launch_stages(f, f->plan[0], dims_mask);
}

// One step into the capture: k_begin, then each dimension's stages on a
// branch of its own (forked from and joined back to the batch's stream) when
// more than one dimension is live.
static int capture_step(FusedSet* f, int mask) {
    if ((mask & (mask - 1)) == 0) return launch_step(f, mask);
    unsigned const g = (unsigned)((f->max_slots + 127) / 128);
    fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 1, f->rotates, f->betas, f->d_work);
    HC_CUDA(cudaEventRecord(f->fork, f->stream));
    for (int d = 0; d < 3; ++d) {
        if (!(mask & (1 << d))) continue;
        HC_CUDA(cudaStreamWaitEvent(f->side[d], f->fork, 0));
        HC_CHECK(launch_stages(f, f->plan[0], 1 << d, f->side[d]));
        HC_CUDA(cudaEventRecord(f->join[d], f->side[d]));
        HC_CUDA(cudaStreamWaitEvent(f->stream, f->join[d], 0));
    }
    return HC_OK;
}

static int capture_graph(FusedSet* f) {
    if (f->graph) { cudaGraphExecDestroy(f->graph); f->graph = nullptr; }
    if (!f->fork) {
        HC_CUDA(cudaEventCreateWithFlags(&f->fork, cudaEventDisableTiming));
        for (int d = 0; d < 3; ++d) {
            HC_CUDA(cudaStreamCreateWithFlags(&f->side[d], cudaStreamNonBlocking));
            HC_CUDA(cudaEventCreateWithFlags(&f->join[d], cudaEventDisableTiming));
        }
    }
    cudaGraph_t g;
    HC_CUDA(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
    int r = capture_step(f, f->graph_dims_mask);
    cudaError_t e = cudaStreamEndCapture(f->stream, &g);
    if (r != HC_OK) { if (e == cudaSuccess) cudaGraphDestroy(g); return r; }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&f->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    f->graph_valid = true;
    return HC_OK;
}

int fused_steps(FusedSet* f, int steps) {
    if (steps <= 0) return HC_OK;
    HC_CHECK(rebuild_items(f));
    if (!f->graph_dims_mask) return HC_OK;
    if (!f->graph_valid) HC_CHECK(capture_graph(f));
    for (int k = 0; k < steps; ++k) HC_CUDA(cudaGraphLaunch(f->graph, f->stream));
    unsigned const g = (unsigned)((f->max_slots + 127) / 128);
    fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 0, f->rotates, f->betas, f->d_work);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_steps_timed(FusedSet* f, int steps, double* stage_ms, int n_stage_ms, double* total_ms) {
    if (steps <= 0) return HC_OK;
    HC_CHECK(rebuild_items(f));
    if (!f->graph_dims_mask) return HC_OK;
    const IntegratorPlan& P = f->plan[0];
    std::vector<cudaEvent_t> ev((size_t)steps * P.n_stages * 2 + 2);
    for (auto& e : ev) HC_CUDA(cudaEventCreate(&e));
    size_t k = 0;
    HC_CUDA(cudaEventRecord(ev[k++], f->stream));
    unsigned const g = (unsigned)((f->max_slots + 127) / 128);
    for (int s = 0; s < steps; ++s) {
        fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 1, f->rotates, f->betas, f->d_work);
        for (int st = 0; st < P.n_stages; ++st) {
            IntegratorPlan one;
            std::memset(&one, 0, sizeof(one));
            one.n_stages = 1;
            one.stage[0] = P.stage[st];
            HC_CUDA(cudaEventRecord(ev[k++], f->stream));
            HC_CHECK(launch_stages(f, one, f->graph_dims_mask));
            HC_CUDA(cudaEventRecord(ev[k++], f->stream));
        }
    }
    fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 0, f->rotates, f->betas, f->d_work);
    HC_CUDA(cudaEventRecord(ev[k++], f->stream));
    HC_CUDA(cudaEventSynchronize(ev[k - 1]));
    size_t j = 1;
    for (int s = 0; s < steps; ++s)
        for (int st = 0; st < P.n_stages; ++st, j += 2) {
            float ms = 0;
            HC_CUDA(cudaEventElapsedTime(&ms, ev[j], ev[j + 1]));
            if (st < n_stage_ms) stage_ms[st] += ms;
        }
    float tot = 0;
    HC_CUDA(cudaEventElapsedTime(&tot, ev[0], ev[k - 1]));
    *total_ms += tot;
    for (auto& e : ev) cudaEventDestroy(e);
    return HC_OK;
}

int fused_step_dt(FusedSet* f, int slot, double dt) {
    HC_CHECK(rebuild_items(f));
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    fz::k_set_dt<<<1, 1, 0, f->stream>>>(f->d_ctl, f->d_inst, slot, dt, 1, f->rotates, f->betas, f->d_work);
    HC_CHECK(launch_stages(f, f->plan[0], 1 << (S.dim - 1)));
    fz::k_set_dt<<<1, 1, 0, f->stream>>>(f->d_ctl, f->d_inst, slot, dt, 0, f->rotates, f->betas, f->d_work);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_num_stages(const FusedSet* f) { return f->plan[0].n_stages; }

// Stage `stage` of one update of one slot with the update's dt: the first
// stage sets the step's coefficients, the last one completes the step (t is
// not advanced, as in fused_step_dt).
int fused_stage(FusedSet* f, int slot, double dt, int stage) {
    HC_CHECK(rebuild_items(f));
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    const IntegratorPlan& P = f->plan[0];
    if (stage < 0 || stage >= P.n_stages) return fail(HC_ERR_INVALID, "stage");
    if (stage == 0) fz::k_set_dt<<<1, 1, 0, f->stream>>>(f->d_ctl, f->d_inst, slot, dt, 1, f->rotates, f->betas, f->d_work);
    IntegratorPlan one;
    std::memset(&one, 0, sizeof(one));
    one.n_stages = 1;
    one.stage[0] = P.stage[stage];
    HC_CHECK(launch_stages(f, one, 1 << (S.dim - 1)));
    if (stage == P.n_stages - 1)
        fz::k_set_dt<<<1, 1, 0, f->stream>>>(f->d_ctl, f->d_inst, slot, dt, 0, f->rotates, f->betas, f->d_work);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

// The two layers next to face (axis, side) of the buffer stage `stage` reads,
// as AoS-6 doubles: read (dir 1: the interior layers next to the face) or
// written (dir 0: the ghost layers beyond it).
int fused_slab(FusedSet* f, int slot, int stage, int axis, int side, int dir, double* host) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    if (axis < 0 || axis >= S.dim || side < 0 || side > 1) return fail(HC_ERR_INVALID, "face");
    if (S.inst.n[axis] < kG) return fail(HC_ERR_INVALID, "the axis has fewer cells than ghost layers");
    const IntegratorPlan& P = f->plan[0];
    int rot = 0;
    if (f->rotates) {
        HC_CUDA(cudaMemcpyAsync(&rot, &f->d_ctl[slot].rot, sizeof(int), cudaMemcpyDeviceToHost, f->stream));
        HC_CUDA(cudaStreamSynchronize(f->stream));
    }
    // slotBuf on the host: a rotated slot sees buffers 0 and rot_buf exchanged
    int const b0 = P.stage[stage].in_buf;
    int const buf = rot ? (b0 == 0 ? f->rot_buf : (b0 == f->rot_buf ? 0 : b0)) : b0;
    long long cells = (long long)kG;
    for (int k = 0; k < S.dim; ++k) if (k != axis) cells *= S.inst.n[k];
    size_t const bytes = (size_t)cells * 6 * sizeof(double);
    HC_CHECK(ensure_staging(f, bytes));
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    if (dir == 0) HC_CUDA(cudaMemcpyAsync(f->staging, host, bytes, cudaMemcpyHostToDevice, f->stream));
    A->slab(f->d_inst, slot, buf, axis, side, dir, static_cast<double*>(f->staging), cells, f->stream);
    HC_CUDA(cudaGetLastError());
    if (dir == 1) HC_CUDA(cudaMemcpyAsync(host, f->staging, bytes, cudaMemcpyDeviceToHost, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    return HC_OK;
}

int fused_calc_dt(FusedSet* f, int slot, double* dt) {
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    if (S.d.fixed_dt > 0) { *dt = S.d.fixed_dt; return HC_OK; }
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    fz::k_reset_dtmin<<<1, 1, 0, f->stream>>>(f->d_ctl, slot);
    A->calc_dt(f->d_inst, f->d_ctl, slot, state_buf(f, slot), f->stream);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaMemcpyAsync(f->h_ctl + slot, f->d_ctl + slot, sizeof(DevCtl), cudaMemcpyDeviceToHost, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    const DevCtl& c = f->h_ctl[slot];
    double m;
    unsigned long long const bits = c.dtmin[c.par];
    std::memcpy(&m, &bits, sizeof(m));
    *dt = S.d.cfl * m;
    return HC_OK;
}

int fused_boundary(FusedSet* f, int slot) {
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    find_aux(f->sch.precision, S.dim)->fill_ghosts(f->d_inst, slot, state_buf(f, slot), f->stream);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int fused_constrain_u(FusedSet* f, int slot) {
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    const AuxLauncher* A = find_aux(f->sch.precision, S.dim);
    A->constrain(f->d_inst, slot, state_buf(f, slot), f->stream);
    A->fill_ghosts(f->d_inst, slot, state_buf(f, slot), f->stream);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

// The per-slot status fields sit at the head of DevCtl; a status read copies
// only those bytes of each slot (one strided copy).
constexpr size_t kStatusBytes = 64;
static_assert(offsetof(DevCtl, rot) + sizeof(int) <= kStatusBytes, "status fields beyond the copied head");
static_assert(offsetof(DevCtl, dtmin) + 2 * sizeof(unsigned long long) <= kStatusBytes, "dtmin beyond the copied head");

int fused_slot_info(FusedSet* f, std::vector<SlotInfo>& out) {
    HC_CUDA(cudaMemcpy2DAsync(f->h_ctl, sizeof(DevCtl), f->d_ctl, sizeof(DevCtl), kStatusBytes, f->max_slots,
                              cudaMemcpyDeviceToHost, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    out.resize(f->max_slots);
    for (int s = 0; s < f->max_slots; ++s) {
        const DevCtl& c = f->h_ctl[s];
        out[s].t = c.t;
        out[s].dt = c.dt;
        out[s].steps = c.steps;
        out[s].active = c.active;
        out[s].done = c.done;
        out[s].status = c.status;
    }
    return HC_OK;
}

int fused_set_time(FusedSet* f, int slot, double t) {
    HC_CUDA(cudaMemcpyAsync(&f->d_ctl[slot].t, &t, sizeof(double), cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    return HC_OK;
}

int fused_set_limits(FusedSet* f, int slot, double t_end, long long max_steps) {
    Slot& S = f->slots[slot];
    S.inst.t_end = t_end;
    S.inst.max_steps = max_steps;
    HC_CUDA(cudaMemcpyAsync(&f->d_inst[slot].t_end, &t_end, sizeof(double), cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaMemcpyAsync(&f->d_inst[slot].max_steps, &max_steps, sizeof(long long), cudaMemcpyHostToDevice, f->stream));
    int const one = 1, zero = 0;
    HC_CUDA(cudaMemcpyAsync(&f->d_ctl[slot].active, &one, sizeof(int), cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaMemcpyAsync(&f->d_ctl[slot].done, &zero, sizeof(int), cudaMemcpyHostToDevice, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    f->items_dirty = true;
    return HC_OK;
}

int fused_conservation(FusedSet* f, int slot, double sums[5]) {
    const Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    double vol = 1.;
    for (int k = 0; k < S.dim; ++k) vol *= S.inst.grid_dx[k];
    int const blocks = 1024;
    find_aux(f->sch.precision, S.dim)->sums(f->d_inst, slot, state_buf(f, slot), vol, f->d_partial, blocks, f->stream);
    HC_CUDA(cudaGetLastError());
    std::vector<double> part(5 * blocks);
    HC_CUDA(cudaMemcpyAsync(part.data(), f->d_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, f->stream));
    HC_CUDA(cudaStreamSynchronize(f->stream));
    for (int j = 0; j < 5; ++j) {
        double sm = 0, c = 0;
        for (int b = 0; b < blocks; ++b) {
            double const y = part[5 * b + j] - c;
            double const t = sm + y;
            c = (t - sm) - y;
            sm = t;
        }
        sums[j] = sm;
    }
    return HC_OK;
}

int fused_stats(FusedSet* f, hc_batch_stats* st) {
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(f, info));
    std::memset(st, 0, sizeof(*st));
    for (int s = 0; s < f->max_slots; ++s) {
        if (!f->slots[s].used) continue;
        st->occupied++;
        st->bytes_in_use += f->slots[s].bytes;
        if (info[s].active) { st->active++; st->cells += f->slots[s].cells; }
    }
    st->tiles = (long long)f->h_nitems[0] + f->h_nitems[1] + f->h_nitems[2];
    st->n_stages = f->plan[0].n_stages;
    for (int d = 0; d < 3; ++d) {
        st->tile[d][0] = f->launcher[d] ? f->launcher[d]->tx : 0;
        st->tile[d][1] = f->launcher[d] ? f->launcher[d]->ty : 0;
        st->tile[d][2] = f->launcher[d] ? f->launcher[d]->tz : 0;
        st->schedule[d] = f->launcher[d] ? f->launcher[d]->variant : 0;
        st->marching[d] = f->launcher[d] ? f->launcher[d]->march : 0;
    }
    return HC_OK;
}

int fused_sync(FusedSet* f) {
    HC_CUDA(cudaStreamSynchronize(f->stream));
    int err = 0;
    HC_CUDA(cudaMemcpy(&err, f->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & DEV_TIMEOUT) return fail(HC_ERR_TIMEOUT, "a bounded wait in the stage kernel ran out");
    return HC_OK;
}

// ---------------------------------------------------------------------------
// autotuner: time whole steps of the live instances with each candidate
// schedule and keep the fastest per dimension
// ---------------------------------------------------------------------------

static std::string tune_key(const FusedSet* f, int dim, long long cells) {
    int bucket = 0;
    while ((1ll << (bucket + 1)) <= cells) ++bucket;
    std::ostringstream o;
    o << "p" << f->sch.precision << "_d" << dim << "_plm" << (f->sch.recon >= HC_RECON_PLM_CONS ? f->sch.recon - 1 : 0) << "_lim"
      << (f->sch.flux_limiter > 0) << "_c" << bucket;
    return o.str();
}

static void reencode_all(FusedSet* f, int dim) {
    cudaStreamSynchronize(f->stream);   // the copies that read the old maps are done
    for (int s = 0; s < f->max_slots; ++s)
        if (f->slots[s].used && f->slots[s].dim == dim) encode_maps(f, s);
    cudaStreamSynchronize(f->stream);
}

int fused_autotune(FusedSet* f, const char* cache_path) {
    std::map<std::string, int> cache;
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream ls(line);
            std::string k;
            int v;
            if (ls >> k >> v) cache[k] = v;
        }
    }
    HC_CUDA(cudaStreamSynchronize(f->stream));
    for (int dim = 1; dim <= 3; ++dim) {
        long long cells = 0;
        for (const Slot& S : f->slots) if (S.used && S.dim == dim) cells += S.cells;
        if (!cells) continue;
        std::string const key = tune_key(f, dim, cells);
        auto it = cache.find(key);
        if (it != cache.end() && find_launcher(f->sch, dim, it->second)) {
            HC_CHECK(set_launcher(f, dim, it->second));
            reencode_all(f, dim);
            f->items_dirty = true;
            f->graph_valid = false;
            continue;
        }
        int best = 0;
        float bestMs = 1e30f;
        std::ostringstream log;
        for (int v = 0; v < kMaxVariants; ++v) {
            if (!find_launcher(f->sch, dim, v)) continue;
            HC_CHECK(set_launcher(f, dim, v));
            reencode_all(f, dim);
            f->items_dirty = true;
            HC_CHECK(rebuild_items(f));
            // whole steps of the live batch (every schedule gives the same
            // bits, so this is plain stepping): one warm-up, `reps` timed
            int const mask = f->graph_dims_mask;
            unsigned const g = (unsigned)((f->max_slots + 127) / 128);
            HC_CHECK(launch_step(f, mask));
            cudaEvent_t e0, e1;
            HC_CUDA(cudaEventCreate(&e0));
            HC_CUDA(cudaEventCreate(&e1));
            cudaEventRecord(e0, f->stream);
            int const reps = 3;
            for (int r = 0; r < reps; ++r) HC_CHECK(launch_step(f, mask));
            cudaEventRecord(e1, f->stream);
            fz::k_begin<<<g, 128, 0, f->stream>>>(f->d_ctl, f->d_inst, f->max_slots, 0, f->rotates, f->betas, f->d_work);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            HC_CUDA(cudaStreamSynchronize(f->stream));
            const StageLauncher* Lc = f->launcher[dim - 1];
            log << "# " << key << " variant " << v << " tile " << Lc->tx << "x" << Lc->ty << "x" << Lc->tz << " threads "
                << Lc->nthreads << " seg " << Lc->seg;
            if (Lc->march) log << " (items: " << f->seg[dim - 1] << ")";
            log << " unroll " << Lc->unroll << " ctas/SM " << Lc->min_ctas
                << " lanes " << Lc->lanes << " slope " << Lc->slope << " ms/step " << ms / reps << "\n";
            if (ms < bestMs) { bestMs = ms; best = v; }
        }
        f->tune_log += log.str();
        HC_CHECK(set_launcher(f, dim, best));
        reencode_all(f, dim);
        f->items_dirty = true;
        f->graph_valid = false;
        cache[key] = best;
    }
    HC_CHECK(rebuild_items(f));
    if (cache_path) {
        std::ofstream out(cache_path);
        for (auto& kv : cache) out << kv.first << " " << kv.second << "\n";
        out << f->tune_log;
    }
    return fused_sync(f);
}

int fused_variant(const FusedSet* f, int dim) { return f->launcher[dim - 1] ? f->launcher[dim - 1]->variant : -1; }

// fused_autotune without advancing one slot's solve (a single solver): its
// state buffer, ghosts included, and its control block are copied aside on the
// device before the timed steps and put back after them.
int fused_autotune_keep(FusedSet* f, int slot, const char* cache_path) {
    Slot& S = f->slots[slot];
    if (!S.used) return fail(HC_ERR_STATE, "slot not in use");
    int const b = state_buf(f, slot);
    size_t const bytes = (size_t)S.inst.plane * 5 * f->esize;
    void* save = nullptr;
    DevCtl* ctl = nullptr;
    HC_CUDA(cudaMalloc(&save, bytes));
    cudaError_t e = cudaMalloc(&ctl, sizeof(DevCtl));
    if (e != cudaSuccess) { cudaFree(save); return cuda_fail(e, "cudaMalloc"); }
    int r = HC_OK;
    e = cudaMemcpyAsync(save, S.inst.buf[b], bytes, cudaMemcpyDeviceToDevice, f->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, f->d_ctl + slot, sizeof(DevCtl), cudaMemcpyDeviceToDevice, f->stream);
    if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync");
    if (r == HC_OK) r = fused_autotune(f, cache_path);
    // put the solve back even if tuning failed part way
    e = cudaMemcpyAsync(S.inst.buf[b], save, bytes, cudaMemcpyDeviceToDevice, f->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(f->d_ctl + slot, ctl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    cudaFree(save);
    cudaFree(ctl);
    if (e != cudaSuccess && r == HC_OK) r = cuda_fail(e, "restoring the solve after tuning");
    f->items_dirty = true;
    return r;
}

int fused_set_schedule(FusedSet* f, int dim, int variant) {
    const StageLauncher* L = find_launcher(f->sch, dim, variant);
    if (!L) return fail(HC_ERR_INVALID, "no such schedule for this scheme and dimension");
    if (f->launcher[dim - 1] == L) return HC_OK;   // already running it (its maps encoded for it)
    HC_CUDA(cudaStreamSynchronize(f->stream));
    HC_CHECK(set_launcher(f, dim, variant));
    reencode_all(f, dim);
    f->items_dirty = true;
    f->graph_valid = false;
    return HC_OK;
}

}  // namespace hc

namespace hc {
namespace fz {
void register_f32_d1(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d2a(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d2b(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d2c(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d2d(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_flux(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_recon(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d2e(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d3b(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d3c(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_d3(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_m2(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_m3(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_m2b(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f32_m2c(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f64_d1(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f64_d2(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);
void register_f64_d3(std::vector<StageLauncher>&, std::vector<AuxLauncher>&);

void register_launchers(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    register_f32_d1(st, aux);
    register_f32_d2a(st, aux);
    register_f32_d2b(st, aux);
    register_f32_d2c(st, aux);
    register_f32_d2d(st, aux);
    register_f32_flux(st, aux);
    register_f32_recon(st, aux);
    register_f32_d2e(st, aux);
    register_f32_d3b(st, aux);
    register_f32_d3c(st, aux);
    register_f32_d3(st, aux);
    register_f32_m2(st, aux);
    register_f32_m3(st, aux);
    register_f32_m2b(st, aux);
    register_f32_m2c(st, aux);
    register_f64_d1(st, aux);
    register_f64_d2(st, aux);
    register_f64_d3(st, aux);
}
}  // namespace fz
}  // namespace hc
