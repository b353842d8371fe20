// hc_api.cu -- the extern "C" entry points declared in include/hydrocuda.h.
#include "hc_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace hc {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? HC_ERR_NOMEM : HC_ERR_CUDA;
}

}  // namespace hc

using namespace hc;

// A context lives until the caller has destroyed it and every solver and
// batch made on it has been destroyed too (one reference each), so handles
// may be released in any order.
struct hc_context {
    int device;
    cudaStream_t stream;
    std::atomic<int> refs{1};
};

static void ctx_retain(hc_context* ctx) { ctx->refs.fetch_add(1); }

static void ctx_release(hc_context* ctx) {
    if (ctx->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

struct hc_solver {
    hc_context* ctx;
    hc_solver_desc d;
    PlainSolver* plain = nullptr;
    FusedSet* fused = nullptr;
    double t = 0;           // plain form: SolverBase.t (a Lua double in the reference)
    long long steps = 0;
    int next_stage = 0;     // fused forms: the stage hc_solver_stage runs next (0: between updates)
    int plain_status = HC_OK;   // plain form: first non-finite dt seen
};

struct hc_batch {
    hc_context* ctx;
    hc_batch_desc d;
    FusedSet* fused = nullptr;
    size_t bytes_in_use = 0;
    std::vector<size_t> slot_bytes;
    std::vector<unsigned long long> tags;
    std::vector<char> used, reported;
};

namespace {

int use_device(const hc_context* ctx) {
    HC_CUDA(cudaSetDevice(ctx->device));
    return HC_OK;
}

int validate_desc(const hc_solver_desc* d) {
    if (!d) return fail(HC_ERR_INVALID, "descriptor is NULL");
    if (d->dim < 1 || d->dim > 3) return fail(HC_ERR_INVALID, "dim must be 1, 2 or 3");
    for (int k = 0; k < d->dim; ++k) {
        if (d->n[k] < 2) return fail(HC_ERR_INVALID, "gridSize must be at least 2 on each active axis");
        if (!(d->maxs[k] > d->mins[k])) return fail(HC_ERR_INVALID, "maxs must exceed mins");
    }
    for (int k = 0; k < 6; ++k)
        if (d->boundary[k] < HC_BOUNDARY_NONE || d->boundary[k] >= HC_NUM_BOUNDARIES)
            return fail(HC_ERR_INVALID, "unknown boundary");
    for (int k = 0; k < d->dim; ++k)
        for (int m = 0; m < 2; ++m)
            if (d->boundary[2 * k + m] == HC_BOUNDARY_QUADRATIC && d->n[k] < 3)
                return fail(HC_ERR_INVALID, "the quadratic boundary extrapolates from 3 interior cells");
    if (d->flux_limiter < 0 || d->flux_limiter >= HC_NUM_LIMITERS) return fail(HC_ERR_INVALID, "unknown flux limiter");
    if (d->slope_limiter < 0 || d->slope_limiter >= HC_NUM_LIMITERS) return fail(HC_ERR_INVALID, "unknown slope limiter");
    if (d->recon < HC_RECON_NONE || d->recon >= HC_NUM_RECONS) return fail(HC_ERR_INVALID, "unknown usePLM");
    if (d->recon != HC_RECON_NONE && d->flux_limiter > 0)
        return fail(HC_ERR_INVALID, "usePLM together with a flux limiter (gridsolver.lua:119 asserts against it)");
    if (d->integrator < 0 || d->integrator >= HC_NUM_INTEGRATORS) return fail(HC_ERR_INVALID, "unknown integrator");
    if (d->precision < HC_F64_PLAIN || d->precision > HC_F32_FUSED) return fail(HC_ERR_INVALID, "unknown precision");
    if (d->flux < 0 || d->flux >= HC_NUM_FLUXES) return fail(HC_ERR_INVALID, "unknown flux");
    if (d->hllc_method < HC_HLLC_DEFAULT || d->hllc_method > HC_HLLC_METHOD_2) return fail(HC_ERR_INVALID, "unknown hllcMethod");
    if (!(d->gamma > 1.)) return fail(HC_ERR_INVALID, "gamma must exceed 1");
    if (!(d->cfl > 0.) && !(d->fixed_dt > 0.)) return fail(HC_ERR_INVALID, "cfl must be positive");
    return HC_OK;
}

long long interior_cells(const hc_solver_desc& d) {
    long long n = 1;
    for (int k = 0; k < d.dim; ++k) n *= d.n[k];
    return n;
}

FusedScheme scheme_of(const hc_solver_desc& d) {
    FusedScheme s;
    s.precision = d.precision;
    s.flux_limiter = d.flux_limiter;
    s.recon = d.recon;
    s.slope_limiter = d.slope_limiter;
    s.integrator = d.integrator;
    s.flux = d.flux;
    s.hllc_method = d.hllc_method;
    return s;
}

}  // namespace

extern "C" {

const char* hc_version(void) { return "0.3"; }

const char* hc_last_error(void) { return g_last_error.c_str(); }

int hc_device_count(int* count) {
    if (!count) return fail(HC_ERR_INVALID, "count is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) { *count = 0; return cuda_fail(e, "cudaGetDeviceCount"); }
    *count = n;
    return HC_OK;
}

int hc_context_create(int device, hc_context** out) {
    if (!out) return fail(HC_ERR_INVALID, "out is NULL");
    int n = 0;
    HC_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(HC_ERR_INVALID, "no such device");
    HC_CUDA(cudaSetDevice(device));
    hc_context* c = new hc_context();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
    *out = c;
    return HC_OK;
}

int hc_context_destroy(hc_context* ctx) {
    if (!ctx) return HC_OK;
    ctx_release(ctx);
    return HC_OK;
}

int hc_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(HC_ERR_INVALID, "out is NULL");
    HC_CUDA(cudaMallocHost(out, bytes));
    return HC_OK;
}

int hc_host_free(void* p) {
    if (p) HC_CUDA(cudaFreeHost(p));
    return HC_OK;
}

// ---- solver ---------------------------------------------------------------

static long long full_cells(const hc_solver_desc& d) {
    long long n = 1;
    for (int k = 0; k < d.dim; ++k) n *= d.n[k] + 4;
    return n;
}

// the interior cells of a ghost-inclusive AoS-6 array (x fastest)
static void copy_interior(const hc_solver_desc& d, const double* full, double* interior) {
    int gs[3], n[3];
    for (int k = 0; k < 3; ++k) {
        n[k] = k < d.dim ? d.n[k] : 1;
        gs[k] = k < d.dim ? d.n[k] + 4 : 1;
    }
    int const g[3] = {d.dim > 0 ? 2 : 0, d.dim > 1 ? 2 : 0, d.dim > 2 ? 2 : 0};
    size_t o = 0;
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j) {
            size_t const src = ((size_t)(k + g[2]) * gs[1] + (j + g[1])) * gs[0] + g[0];
            std::memcpy(interior + o * 6, full + src * 6, (size_t)n[0] * 6 * sizeof(double));
            o += (size_t)n[0];
        }
}

int hc_solver_create(hc_context* ctx, const hc_solver_desc* desc, hc_solver** out) {
    if (!ctx || !out) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(validate_desc(desc));
    HC_CHECK(use_device(ctx));
    hc_solver* s = new hc_solver();
    s->ctx = ctx;
    ctx_retain(ctx);
    s->d = *desc;
    int r;
    if (desc->precision == HC_F64_PLAIN) {
        r = plain_create(*desc, ctx->stream, &s->plain);
    } else {
        r = fused_create(scheme_of(*desc), 1, ctx->stream, &s->fused);
        if (r == HC_OK) r = fused_add(s->fused, 0, *desc, nullptr, HC_LAYOUT_AOS6_F64, INFINITY, LLONG_MAX, 0);
    }
    if (r != HC_OK) {
        std::string const msg = g_last_error;
        hc_solver_destroy(s);
        g_last_error = msg;
        return r;
    }
    *out = s;
    return HC_OK;
}

int hc_solver_destroy(hc_solver* s) {
    if (!s) return HC_OK;
    cudaSetDevice(s->ctx->device);
    if (s->plain) plain_destroy(s->plain);
    if (s->fused) fused_destroy(s->fused);
    hc_context* const ctx = s->ctx;
    delete s;
    ctx_release(ctx);
    return HC_OK;
}

int hc_solver_reset_state(hc_solver* s, const void* cons, int layout) {
    if (!s || !cons) return fail(HC_ERR_INVALID, "NULL argument");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) {
        HC_CHECK(plain_set_interior(s->plain, cons, layout));
        HC_CHECK(plain_boundary(s->plain));
        HC_CHECK(plain_constrain_u(s->plain));
        s->t = 0;
        s->steps = 0;
        HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
        return HC_OK;
    }
    HC_CHECK(fused_set_state(s->fused, 0, cons, layout, 1));
    return fused_sync(s->fused);
}

int hc_solver_init_state(hc_solver* s, const hc_init* init) {
    if (!s || !init) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    HC_CHECK(init_validate(*init, s->d));
    if (s->plain) {
        HC_CHECK(plain_init_state(s->plain, *init, s->d));
        HC_CHECK(plain_boundary(s->plain));
        HC_CHECK(plain_constrain_u(s->plain));
        s->t = 0;
        s->steps = 0;
        HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
        return HC_OK;
    }
    HC_CHECK(fused_init_state(s->fused, 0, *init));
    return fused_sync(s->fused);
}

int hc_solver_set_state(hc_solver* s, const void* cons, int layout, int with_ghosts) {
    if (!s || !cons) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    if (with_ghosts) {
        if (layout != HC_LAYOUT_AOS6_F64) return fail(HC_ERR_INVALID, "ghost-inclusive state I/O is AOS6_F64");
        if (s->plain) return plain_set_full(s->plain, (const double*)cons);
        // the fused forms take the interior; their ghosts follow from the boundary
        std::vector<double> in((size_t)interior_cells(s->d) * 6);
        copy_interior(s->d, static_cast<const double*>(cons), in.data());
        HC_CHECK(fused_set_state(s->fused, 0, in.data(), HC_LAYOUT_AOS6_F64, 0));
        return fused_sync(s->fused);
    }
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    if (s->plain) return plain_set_interior(s->plain, cons, layout);
    HC_CHECK(fused_set_state(s->fused, 0, cons, layout, 0));
    return fused_sync(s->fused);
}

int hc_solver_get_state(hc_solver* s, void* cons, int layout, int with_ghosts) {
    if (!s || !cons) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    if (with_ghosts) {
        if (layout != HC_LAYOUT_AOS6_F64) return fail(HC_ERR_INVALID, "ghost-inclusive state I/O is AOS6_F64");
        if (s->plain) return plain_get_full(s->plain, (double*)cons);
        // the fused forms: the interior, expanded to the reference's UBuf by its boundary rules
        size_t const nin = (size_t)interior_cells(s->d), nfull = (size_t)full_cells(s->d);
        void* tmp = nullptr;
        HC_CUDA(cudaMalloc(&tmp, (nin + nfull) * 6 * sizeof(double)));
        double* interior = static_cast<double*>(tmp);
        double* full = interior + nin * 6;
        int r = fused_get_state_dev(s->fused, 0, interior, HC_LAYOUT_AOS6_F64);
        if (r == HC_OK) r = plain_expand_full(s->d, interior, HC_LAYOUT_AOS6_F64, full, s->ctx->stream);
        if (r == HC_OK) {
            cudaError_t e = cudaMemcpyAsync(cons, full, nfull * 6 * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
            if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync");
        }
        cudaFree(tmp);
        return r;
    }
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    if (s->plain) return plain_get_interior(s->plain, cons, layout);
    return fused_get_state(s->fused, 0, cons, layout);
}

// ---- headless visualisation ---------------------------------------------------

// The solver's interior state as AoS-6 FP64 on the device: the plain form's
// UBuf in place, the fused forms through a scratch copy (*scratch, freed by
// the caller).
static int viz_state(hc_solver* s, VizState& st, void** scratch) {
    *scratch = nullptr;
    st.d = s->d;
    long long n[3], f[3];
    for (int k = 0; k < 3; ++k) {
        n[k] = k < s->d.dim ? s->d.n[k] : 1;
        f[k] = k < s->d.dim ? n[k] + 4 : 1;
    }
    if (s->plain) {
        st.stride[0] = 1;
        st.stride[1] = f[0];
        st.stride[2] = f[0] * f[1];
        long long off = 0;
        for (int k = 0; k < s->d.dim; ++k) off += 2 * st.stride[k];
        st.U = plain_state_dev(s->plain) + 6 * off;
        return HC_OK;
    }
    HC_CUDA(cudaMalloc(scratch, (size_t)interior_cells(s->d) * 6 * sizeof(double)));
    st.U = static_cast<const double*>(*scratch);
    st.stride[0] = 1;
    st.stride[1] = n[0];
    st.stride[2] = n[0] * n[1];
    return fused_get_state_dev(s->fused, 0, *scratch, HC_LAYOUT_AOS6_F64);
}

int hc_solver_display(hc_solver* s, int var, int zero_border, double* out) {
    if (!s || !out) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    VizState st;
    void* scratch = nullptr;
    double* dev = nullptr;
    size_t const bytes = (size_t)full_cells(s->d) * sizeof(double);
    int r = viz_state(s, st, &scratch);
    if (r == HC_OK) {
        cudaError_t e = cudaMalloc(&dev, bytes);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMalloc");
    }
    if (r == HC_OK) r = viz_display(st, var, zero_border, dev, s->ctx->stream);
    if (r == HC_OK) {
        cudaError_t e = cudaMemcpyAsync(out, dev, bytes, cudaMemcpyDeviceToHost, s->ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync");
    }
    cudaFree(dev);
    cudaFree(scratch);
    return r;
}

int hc_solver_display_range(hc_solver* s, int var, double out[4]) {
    if (!s || !out) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    VizState st;
    void* scratch = nullptr;
    int r = viz_state(s, st, &scratch);
    if (r == HC_OK) r = viz_range(st, var, out, s->ctx->stream);
    cudaFree(scratch);
    return r;
}

int hc_solver_render(hc_solver* s, const hc_render* rr, unsigned char* rgba) {
    if (!s || !rr || !rgba) return fail(HC_ERR_INVALID, "NULL argument");
    if (rr->width <= 0 || rr->height <= 0 || (long long)rr->width * rr->height > (1ll << 28))
        return fail(HC_ERR_INVALID, "image size");
    HC_CHECK(use_device(s->ctx));
    VizState st;
    void* scratch = nullptr;
    void* img = nullptr;
    size_t const bytes = (size_t)rr->width * rr->height * 4;
    int r = viz_state(s, st, &scratch);
    if (r == HC_OK) {
        cudaError_t e = cudaMalloc(&img, bytes);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMalloc");
    }
    if (r == HC_OK) r = viz_render(st, *rr, static_cast<unsigned char*>(img), s->ctx->stream);
    if (r == HC_OK) {
        cudaError_t e = cudaMemcpyAsync(rgba, img, bytes, cudaMemcpyDeviceToHost, s->ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync");
    }
    cudaFree(img);
    cudaFree(scratch);
    return r;
}

int hc_solver_boundary(hc_solver* s) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) HC_CHECK(plain_boundary(s->plain));
    else HC_CHECK(fused_boundary(s->fused, 0));
    HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return HC_OK;
}

int hc_solver_constrain_u(hc_solver* s) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) HC_CHECK(plain_constrain_u(s->plain));
    else HC_CHECK(fused_constrain_u(s->fused, 0));
    HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return HC_OK;
}

int hc_solver_calc_dt(hc_solver* s, double* dt) {
    if (!s || !dt) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) return plain_calc_dt(s->plain, s->d.cfl, s->d.fixed_dt, dt);
    return fused_calc_dt(s->fused, 0, dt);
}

int hc_solver_step(hc_solver* s, double dt) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (s->next_stage) return fail(HC_ERR_STATE, "an update run stage by stage is in progress");
    if (!(dt >= 0) || !std::isfinite(dt)) return fail(HC_ERR_INVALID, "dt must be finite and non-negative");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) {
        HC_CHECK(plain_step(s->plain, s->d.integrator, dt));
        HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
        return HC_OK;
    }
    HC_CHECK(fused_step_dt(s->fused, 0, dt));
    return fused_sync(s->fused);
}

static int solver_status(hc_solver* s) {
    if (s->plain) return s->plain_status == HC_OK ? HC_OK : fail(s->plain_status, "calcDT produced a non-finite dt");
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(s->fused, info));
    if (info[0].status & DEV_TIMEOUT) return fail(HC_ERR_TIMEOUT, "a bounded device wait ran out");
    if (info[0].status & DEV_NONFINITE) return fail(HC_ERR_NONFINITE, "the solve produced a non-finite state or dt");
    return HC_OK;
}

int hc_solver_stage(hc_solver* s, double dt) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (!(dt >= 0) || !std::isfinite(dt)) return fail(HC_ERR_INVALID, "dt must be finite and non-negative");
    if (s->plain) return fail(HC_ERR_INVALID, "the plain form steps whole updates (hc_solver_step)");
    HC_CHECK(use_device(s->ctx));
    HC_CHECK(fused_stage(s->fused, 0, dt, s->next_stage));
    s->next_stage = (s->next_stage + 1) % fused_num_stages(s->fused);
    return fused_sync(s->fused);
}

int hc_solver_autotune(hc_solver* s, const char* cache_path) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (s->plain) return HC_OK;   // one kernel set: nothing to choose
    if (s->next_stage) return fail(HC_ERR_STATE, "an update run stage by stage is in progress");
    HC_CHECK(use_device(s->ctx));
    return fused_autotune_keep(s->fused, 0, cache_path);
}

int hc_solver_num_stages(hc_solver* s, int* n) {
    if (!s || !n) return fail(HC_ERR_INVALID, "NULL argument");
    if (s->plain) return fail(HC_ERR_INVALID, "the plain form steps whole updates (hc_solver_step)");
    *n = fused_num_stages(s->fused);
    return HC_OK;
}

static int solver_slab(hc_solver* s, int axis, int side, double* buf, int dir) {
    if (!s || !buf) return fail(HC_ERR_INVALID, "NULL argument");
    if (s->plain) return fail(HC_ERR_INVALID, "the plain form steps whole updates: slabs are for the fused forms");
    HC_CHECK(use_device(s->ctx));
    return fused_slab(s->fused, 0, s->next_stage, axis, side, dir, buf);
}

int hc_solver_get_slab(hc_solver* s, int axis, int side, double* out) { return solver_slab(s, axis, side, out, 1); }

int hc_solver_set_slab(hc_solver* s, int axis, int side, const double* in) {
    return solver_slab(s, axis, side, const_cast<double*>(in), 0);
}

int hc_solver_update(hc_solver* s, double* dt_out) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (s->next_stage) return fail(HC_ERR_STATE, "an update run stage by stage is in progress");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) {
        double dt;
        HC_CHECK(plain_calc_dt(s->plain, s->d.cfl, s->d.fixed_dt, &dt));
        // the reference prints "got a bad dt" and steps on (solverbase.lua:3017-3019)
        if (!std::isfinite(dt)) s->plain_status = HC_ERR_NONFINITE;
        HC_CHECK(plain_step(s->plain, s->d.integrator, dt));
        s->t = s->t + dt;
        s->steps += 1;
        HC_CHECK(plain_boundary(s->plain));
        HC_CUDA(cudaStreamSynchronize(s->ctx->stream));
        if (dt_out) *dt_out = dt;
        return HC_OK;
    }
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(s->fused, info));
    HC_CHECK(fused_set_limits(s->fused, 0, INFINITY, info[0].steps + 1));
    HC_CHECK(fused_steps(s->fused, 1));
    HC_CHECK(fused_sync(s->fused));
    HC_CHECK(fused_slot_info(s->fused, info));
    if (dt_out) *dt_out = info[0].dt;
    return HC_OK;
}

int hc_solver_run_until(hc_solver* s, double t_end, long long max_steps, long long* steps_done) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (max_steps < 0) return fail(HC_ERR_INVALID, "max_steps");
    HC_CHECK(use_device(s->ctx));
    long long n = 0;
    if (s->plain) {
        while (!(s->t >= t_end) && n < max_steps) {
            HC_CHECK(hc_solver_update(s, nullptr));
            ++n;
            if (!std::isfinite(s->t)) break;   // t can no longer reach t_end
        }
        if (steps_done) *steps_done = n;
        return std::isfinite(s->t) ? HC_OK : fail(HC_ERR_NONFINITE, "time became non-finite");
    }
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(s->fused, info));
    long long const start = info[0].steps;
    long long const limit = max_steps > LLONG_MAX - start ? LLONG_MAX : start + max_steps;
    HC_CHECK(fused_set_limits(s->fused, 0, t_end, limit));
    int chunk = 4;
    for (;;) {
        HC_CHECK(fused_steps(s->fused, chunk));
        HC_CHECK(fused_sync(s->fused));
        HC_CHECK(fused_slot_info(s->fused, info));
        if (!info[0].active || info[0].done) break;
        if (chunk < 64) chunk *= 2;
    }
    if (steps_done) *steps_done = info[0].steps - start;
    return std::isfinite(info[0].t) ? HC_OK : fail(HC_ERR_NONFINITE, "time became non-finite");
}

int hc_solver_get_time(hc_solver* s, double* t) {
    if (!s || !t) return fail(HC_ERR_INVALID, "NULL argument");
    if (s->plain) { *t = s->t; return HC_OK; }
    HC_CHECK(use_device(s->ctx));
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(s->fused, info));
    *t = info[0].t;
    return HC_OK;
}

int hc_solver_set_time(hc_solver* s, double t) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    if (s->plain) { s->t = t; return HC_OK; }
    HC_CHECK(use_device(s->ctx));
    return fused_set_time(s->fused, 0, t);
}

int hc_solver_conservation(hc_solver* s, double sums[5]) {
    if (!s || !sums) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(s->ctx));
    if (s->plain) return plain_conservation(s->plain, sums);
    return fused_conservation(s->fused, 0, sums);
}

int hc_solver_status(hc_solver* s) {
    if (!s) return fail(HC_ERR_INVALID, "NULL solver");
    HC_CHECK(use_device(s->ctx));
    return solver_status(s);
}

// ---- batch ------------------------------------------------------------------

int hc_batch_create(hc_context* ctx, const hc_batch_desc* desc, hc_batch** out) {
    if (!ctx || !desc || !out) return fail(HC_ERR_INVALID, "NULL argument");
    if (desc->precision != HC_F32_FUSED && desc->precision != HC_F64_FUSED)
        return fail(HC_ERR_INVALID, "a batch runs the fused form (HC_F32_FUSED or HC_F64_FUSED)");
    if (desc->max_slots <= 0 || desc->max_slots > (1 << 20)) return fail(HC_ERR_INVALID, "max_slots");
    HC_CHECK(use_device(ctx));
    FusedScheme sch;
    sch.precision = desc->precision;
    sch.flux_limiter = desc->flux_limiter;
    sch.recon = desc->recon;
    sch.slope_limiter = desc->slope_limiter;
    sch.integrator = desc->integrator;
    sch.flux = desc->flux;
    sch.hllc_method = desc->hllc_method;
    if (desc->flux < 0 || desc->flux >= HC_NUM_FLUXES) return fail(HC_ERR_INVALID, "unknown flux");
    if (desc->hllc_method < HC_HLLC_DEFAULT || desc->hllc_method > HC_HLLC_METHOD_2)
        return fail(HC_ERR_INVALID, "unknown hllcMethod");
    hc_batch* b = new hc_batch();
    b->ctx = ctx;
    b->d = *desc;
    int const r = fused_create(sch, desc->max_slots, ctx->stream, &b->fused);
    if (r != HC_OK) { delete b; return r; }
    ctx_retain(ctx);
    b->slot_bytes.assign(desc->max_slots, 0);
    b->tags.assign(desc->max_slots, 0);
    b->used.assign(desc->max_slots, 0);
    b->reported.assign(desc->max_slots, 0);
    *out = b;
    return HC_OK;
}

int hc_batch_destroy(hc_batch* b) {
    if (!b) return HC_OK;
    cudaSetDevice(b->ctx->device);
    fused_destroy(b->fused);
    hc_context* const ctx = b->ctx;
    delete b;
    ctx_release(ctx);
    return HC_OK;
}

// The checks of an admission and the slot it would take (not yet marked).
static int admit_check(hc_batch* b, const hc_solver_desc* desc, const hc_init* init, int layout, size_t extra_bytes,
                       size_t* bytes, int* slot) {
    HC_CHECK(validate_desc(desc));
    if (init) HC_CHECK(init_validate(*init, *desc));
    if (desc->recon != b->d.recon || desc->slope_limiter != b->d.slope_limiter || desc->flux_limiter != b->d.flux_limiter ||
        desc->integrator != b->d.integrator || desc->flux != b->d.flux || desc->hllc_method != b->d.hllc_method)
        return fail(HC_ERR_INVALID, "the instance's scheme differs from the batch's");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    *bytes = fused_instance_bytes(b->fused, *desc);
    if (b->bytes_in_use + extra_bytes + *bytes > b->d.hbm_budget)
        return fail(HC_ERR_BUDGET, "admission would exceed the batch's HBM budget");
    int s = -1;
    for (int k = 0; k < b->d.max_slots; ++k)
        if (!b->used[k]) { s = k; break; }
    if (s < 0) return fail(HC_ERR_NO_SLOT, "every slot is in use");
    *slot = s;
    return HC_OK;
}

static void admit_commit(hc_batch* b, int s, size_t bytes, unsigned long long tag) {
    b->used[s] = 1;
    b->reported[s] = 0;
    b->tags[s] = tag;
    b->slot_bytes[s] = bytes;
    b->bytes_in_use += bytes;
}

static int batch_admit(hc_batch* b, const hc_solver_desc* desc, const void* cons, int layout, const hc_init* init,
                       double t_end, long long max_steps, unsigned long long tag, int* slot, int sync = 1) {
    if (!b || !desc || !(cons || init) || !slot) return fail(HC_ERR_INVALID, "NULL argument");
    if (max_steps <= 0) max_steps = LLONG_MAX;
    HC_CHECK(use_device(b->ctx));
    size_t bytes = 0;
    int s = -1;
    HC_CHECK(admit_check(b, desc, init, layout, 0, &bytes, &s));
    HC_CHECK(fused_add(b->fused, s, *desc, cons, layout, t_end, max_steps, 1, init, sync));
    admit_commit(b, s, bytes, tag);
    *slot = s;
    return HC_OK;
}

int hc_batch_admit(hc_batch* b, const hc_solver_desc* desc, const void* cons, int layout,
                   double t_end, long long max_steps, unsigned long long tag, int* slot) {
    if (!cons) return fail(HC_ERR_INVALID, "NULL argument");
    return batch_admit(b, desc, cons, layout, nullptr, t_end, max_steps, tag, slot);
}

int hc_batch_admit_init(hc_batch* b, const hc_solver_desc* desc, const hc_init* init,
                        double t_end, long long max_steps, unsigned long long tag, int* slot) {
    if (!init) return fail(HC_ERR_INVALID, "NULL argument");
    // no host buffer is read after return: the set-up launches stay queued
    // behind whatever the batch's stream is running
    return batch_admit(b, desc, nullptr, HC_LAYOUT_AOS6_F64, init, t_end, max_steps, tag, slot, 0);
}

int hc_batch_admit_many(hc_batch* b, int count, const hc_solver_desc* descs, const void* const* cons, int layout,
                        const double* t_end, const long long* max_steps, const unsigned long long* tags,
                        int* slots, int* n_admitted) {
    if (!b || count < 0 || (count > 0 && (!descs || !cons || !slots)) || !n_admitted)
        return fail(HC_ERR_INVALID, "NULL argument");
    *n_admitted = 0;
    for (int k = 0; k < count; ++k) slots[k] = -1;
    HC_CHECK(use_device(b->ctx));
    // every check first (slots taken in turn, the budget summed), then the
    // accepted ones in one pass of the fused set
    int r = HC_OK;
    std::vector<size_t> bytes;
    std::vector<double> te;
    std::vector<long long> ms;
    size_t extra = 0;
    int n = 0;
    for (; n < count; ++n) {
        if (!cons[n]) { r = fail(HC_ERR_INVALID, "NULL argument"); break; }
        size_t by = 0;
        int s = -1;
        r = admit_check(b, &descs[n], nullptr, layout, extra, &by, &s);
        if (r != HC_OK) break;
        b->used[s] = 1;   // taken for the following searches
        slots[n] = s;
        bytes.push_back(by);
        extra += by;
        te.push_back(t_end ? t_end[n] : INFINITY);
        ms.push_back(max_steps && max_steps[n] > 0 ? max_steps[n] : LLONG_MAX);
    }
    for (int k = 0; k < n; ++k) b->used[slots[k]] = 0;
    int done = 0;
    int ra = n ? fused_add_many(b->fused, n, slots, descs, cons, layout, te.data(), ms.data(), 1, &done) : HC_OK;
    for (int k = 0; k < done; ++k) admit_commit(b, slots[k], bytes[k], tags ? tags[k] : (unsigned long long)k);
    for (int k = done; k < count; ++k) slots[k] = -1;
    *n_admitted = done;
    if (ra != HC_OK && r == HC_OK) r = ra;
    // the host buffers are not read after return
    int const rs = fused_sync(b->fused);
    return r != HC_OK ? r : rs;
}

int hc_batch_step(hc_batch* b, int steps, int* n_active) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    HC_CHECK(use_device(b->ctx));
    HC_CHECK(fused_steps(b->fused, steps));
    HC_CHECK(fused_sync(b->fused));
    if (n_active) {
        std::vector<SlotInfo> info;
        HC_CHECK(fused_slot_info(b->fused, info));
        int n = 0;
        for (int k = 0; k < b->d.max_slots; ++k) n += b->used[k] && info[k].active;
        *n_active = n;
    }
    return HC_OK;
}

int hc_batch_step_async(hc_batch* b, int steps) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    HC_CHECK(use_device(b->ctx));
    return fused_steps(b->fused, steps);
}

int hc_batch_wait(hc_batch* b, int* n_active) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    HC_CHECK(use_device(b->ctx));
    HC_CHECK(fused_sync(b->fused));
    if (n_active) {
        std::vector<SlotInfo> info;
        HC_CHECK(fused_slot_info(b->fused, info));
        int n = 0;
        for (int k = 0; k < b->d.max_slots; ++k) n += b->used[k] && info[k].active;
        *n_active = n;
    }
    return HC_OK;
}

int hc_batch_step_timed(hc_batch* b, int steps, double* stage_ms, int n_stage_ms, double* total_ms) {
    if (!b || !total_ms || (n_stage_ms > 0 && !stage_ms)) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(b->ctx));
    HC_CHECK(fused_steps_timed(b->fused, steps, stage_ms, n_stage_ms, total_ms));
    return fused_sync(b->fused);
}

int hc_batch_list(hc_batch* b, hc_done* out, int cap, int* n_out) {
    if (!b || !n_out || (cap > 0 && !out)) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(b->ctx));
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(b->fused, info));
    int n = 0;
    for (int k = 0; k < b->d.max_slots && n < cap; ++k) {
        if (!b->used[k]) continue;
        out[n].slot = k;
        out[n].status = info[k].status ? (info[k].status & DEV_TIMEOUT ? HC_ERR_TIMEOUT : HC_ERR_NONFINITE) : HC_OK;
        out[n].tag = b->tags[k];
        out[n].steps = info[k].steps;
        out[n].t = info[k].t;
        ++n;
    }
    *n_out = n;
    return HC_OK;
}

int hc_batch_poll(hc_batch* b, hc_done* out, int cap, int* n_out) {
    if (!b || !n_out || (cap > 0 && !out)) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(b->ctx));
    std::vector<SlotInfo> info;
    HC_CHECK(fused_slot_info(b->fused, info));
    int n = 0;
    for (int k = 0; k < b->d.max_slots && n < cap; ++k) {
        if (!b->used[k] || b->reported[k] || !info[k].done) continue;
        out[n].slot = k;
        out[n].status = info[k].status ? (info[k].status & DEV_TIMEOUT ? HC_ERR_TIMEOUT : HC_ERR_NONFINITE) : HC_OK;
        out[n].tag = b->tags[k];
        out[n].steps = info[k].steps;
        out[n].t = info[k].t;
        b->reported[k] = 1;
        ++n;
    }
    *n_out = n;
    return HC_OK;
}

int hc_batch_fetch(hc_batch* b, int slot, void* cons, int layout) {
    if (!b || !cons) return fail(HC_ERR_INVALID, "NULL argument");
    if (slot < 0 || slot >= b->d.max_slots || !b->used[slot]) return fail(HC_ERR_STATE, "slot not in use");
    HC_CHECK(use_device(b->ctx));
    return fused_get_state(b->fused, slot, cons, layout);
}

int hc_batch_fetch_many(hc_batch* b, int count, const int* slots, void* const* cons, int layout) {
    if (!b || count < 0 || (count > 0 && (!slots || !cons))) return fail(HC_ERR_INVALID, "NULL argument");
    if (layout < 0 || layout > 2) return fail(HC_ERR_INVALID, "layout");
    for (int k = 0; k < count; ++k) {
        if (!cons[k]) return fail(HC_ERR_INVALID, "NULL argument");
        if (slots[k] < 0 || slots[k] >= b->d.max_slots || !b->used[slots[k]]) return fail(HC_ERR_STATE, "slot not in use");
    }
    HC_CHECK(use_device(b->ctx));
    int const r = count ? fused_get_state_many(b->fused, count, slots, cons, layout) : HC_OK;
    int const rs = fused_sync(b->fused);
    return r != HC_OK ? r : rs;
}

int hc_batch_retire(hc_batch* b, int slot) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    if (slot < 0 || slot >= b->d.max_slots || !b->used[slot]) return fail(HC_ERR_STATE, "slot not in use");
    HC_CHECK(use_device(b->ctx));
    HC_CHECK(fused_remove(b->fused, slot));
    b->used[slot] = 0;
    b->bytes_in_use -= b->slot_bytes[slot];
    b->slot_bytes[slot] = 0;
    return HC_OK;
}

int hc_batch_stats_get(hc_batch* b, hc_batch_stats* st) {
    if (!b || !st) return fail(HC_ERR_INVALID, "NULL argument");
    HC_CHECK(use_device(b->ctx));
    return fused_stats(b->fused, st);
}

int hc_batch_conservation(hc_batch* b, int slot, double sums[5]) {
    if (!b || !sums) return fail(HC_ERR_INVALID, "NULL argument");
    if (slot < 0 || slot >= b->d.max_slots || !b->used[slot]) return fail(HC_ERR_STATE, "slot not in use");
    HC_CHECK(use_device(b->ctx));
    return fused_conservation(b->fused, slot, sums);
}

int hc_batch_autotune(hc_batch* b, const char* cache_path) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    HC_CHECK(use_device(b->ctx));
    return fused_autotune(b->fused, cache_path);
}

int hc_batch_set_schedule(hc_batch* b, int dim, int variant) {
    if (!b) return fail(HC_ERR_INVALID, "NULL batch");
    if (dim < 1 || dim > 3) return fail(HC_ERR_INVALID, "dim must be 1, 2 or 3");
    HC_CHECK(use_device(b->ctx));
    return fused_set_schedule(b->fused, dim, variant);
}

}  // extern "C"
