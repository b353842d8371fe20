// hc_fused.cuh -- the fused stage kernel: one launch per Runge-Kutta stage
// replaces the reference's boundary / calcLR / calcFlux / calcDerivFromFlux /
// multAdd / constrainU / calcDT sequence for every tile of every instance.
//
// Layout in HBM: per instance and per state buffer, 5 structure-of-arrays
// planes (rho, m.x, m.y, m.z, ETotal) of the padded grid (numGhost = 2 ghost
// layers on each active axis, rows padded to 32 elements).  ePot is always 0
// for these problems and is not stored.
//
// Per tile (TX x TY x TZ interior cells) a CTA:
//   1. stages the tile plus its 2-cell halo (a (TX+4)(TY+4)(TZ+4) x 5 box)
//      into shared memory with one TMA tensor load (cp.async.bulk.tensor,
//      mbarrier completion, bounded wait);
//   2. sweeps every axis but the last with one thread per line segment of L
//      cells: a register window slides along the segment, computing each
//      cell's PLM slope once and each interface's Roe flux once, and writes
//      the flux difference of each cell into a shared-memory accumulator
//      (calcDerivFromFlux: deriv = ((0 - X) - Y) - Z);
//   3. sweeps the last axis the same way, and as each cell's last face flux
//      is known, finishes the cell: Runge-Kutta combination
//      (u = sum alpha_k u^(k) + dt sum beta_k L(u^(k)), terms in the
//      reference's order), constrainU, the store, the ghost copies the
//      boundary condition maps to this cell (the boundary fill becomes a
//      scatter, so no separate boundary launch exists), and on the last stage
//      the cell's CFL dt, reduced by warp shuffles into one FP64 atomicMin
//      per warp.
//
// Two arithmetic forms share this code: EXACT (double, the reference's
// literal expressions from hc_ref_math.cuh, compiled without FMA
// contraction) and fast (hc_fast_math.cuh, any precision).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "hc_internal.h"
#include "hc_ref_math.cuh"
#include "hc_fast_math.cuh"
#include "hc_lanes.cuh"

namespace hc {
namespace fz {

constexpr int kMaxBufs = 4;      // state buffers per instance
constexpr int kMaxDBufs = 4;     // stored-derivative buffers per instance
constexpr int kG = 2;            // numGhost
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

struct DevInst {
    int dim;
    int n[3];              // interior extents (1 on unused axes)
    int px, py, pz;        // padded extents; px is the row pitch in elements
    long long plane;       // elements per field plane
    int bc[6];
    double grid_dx[3];
    double area[3];        // areaL * invVolume of calcDerivFromFlux, per side
    int skipDeriv[3];      // volume <= 1e-7: the side adds nothing
    int zeroFlux[3];       // area <= 1e-7: calcFlux writes a zero flux
    double gamma, rhoMin, PMin, cfl, fixed_dt, t_end;
    long long max_steps;
    int stop_on_error;     // 1 (batched solves): a non-finite state or dt ends the instance
    // the same constants in FP32, converted once on the host
    float f_gamma, f_g1, f_rhoMin, f_PMin, f_invg1, f_area[3], f_gdx[3];
    int entropyFix;            // Roe: useEntropyFluxFix with entropyFactor (f_: 0 when off)
    double entropyFactor;
    float f_entropyFactor;
    double fixedCons[6][5];    // HC_BOUNDARY_FIXED sides: the ghost cells' state
    void* buf[kMaxBufs];
    void* dbuf[kMaxDBufs];
};

struct DevCtl {
    double t, dt;
    unsigned long long dtmin[2];   // FP64 bits of the CFL min (positive: order-preserving)
    long long steps;
    int active, stepping, done, status, par;
    int rot;                       // 1: state buffers 0 and StageArgs::rot_buf are swapped for this slot
    // per-step coefficients, set when a step begins: beta * dt of each stage
    // ([stage][term], term 4 = the stage's own derivative), dt / grid_dx
    double cb_d[4][5];
    float cb_f[4][5];
    double dtdx_d[3];
    float dtdx_f[3];
};

// beta coefficients of the integrator plan, [stage][term] as in DevCtl::cb_*
struct BetaTable {
    double b[4][5];
};

__device__ __forceinline__ void fillStepCoefs(DevCtl& c, const DevInst& I, const BetaTable& bt, double dt) {
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            c.cb_d[s][m] = bt.b[s][m] * dt;
            c.cb_f[s][m] = (float)c.cb_d[s][m];
        }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c.dtdx_d[d] = dt / I.grid_dx[d];
        c.dtdx_f[d] = (float)c.dtdx_d[d];
    }
}

struct StageDev {
    int stage;
    int in_buf, out_buf;
    int n_alpha;
    int alpha_buf[4];
    double alpha[4];
    float alpha_f[4];
    int n_beta;
    int beta_buf[4];
    double beta[4];
    double beta_cur;
    int store_deriv;
    int last;
};

struct StageArgs {
    const DevInst* inst;
    DevCtl* ctl;
    const CUtensorMap* tmaps;   // [slot * kMaxBufs + buf]
    const int4* items;          // {slot, tile x, tile y, tile z}
    const int* nitems;
    StageDev st;
    int rot_buf;                // result buffer of a rotating plan (0: the plan does not rotate)
    int* err;
    int flux;                   // HC_FLUX_*
    int hllcMethod;             // euler-hllc's hllcMethod, 0..2
    int recon;                  // HC_RECON_*
    int* work;                  // marching kernels: this launch's work counter (zeroed when the step begins)
    int force_timeout;          // test knob, 0 in normal use: the first wait for each copy counts as run out
    const int* seg;             // marching kernels: rows (2D) / planes (3D) per segment of the item list
};

// Work counters of the marching kernels: one per (stage, dimension), zeroed by
// the kernel that begins a step.
constexpr int kWorkCounters = 4 * 3;

// A slot whose step count left its state in the other buffer of a rotating
// plan (forward Euler) sees buffers 0 and rot_buf exchanged.
__device__ __forceinline__ int slotBuf(int b, int rot, int r) {
    return rot ? (b == 0 ? r : (b == r ? 0 : b)) : b;
}

// ---------------------------------------------------------------------------
// TMA / mbarrier
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after `limit` polls (each poll may itself suspend
// for a short, hardware-chosen time).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned phase, unsigned limit) {
    for (unsigned i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

template <int RANK>
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, uint64_t* bar) {
    uint64_t const m = reinterpret_cast<uint64_t>(map);
    if (RANK == 2) {
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
            ::"r"(smem_u32(dst)), "l"(m), "r"(c0), "r"(c1), "r"(smem_u32(bar)) : "memory");
    } else if (RANK == 3) {
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
            ::"r"(smem_u32(dst)), "l"(m), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar)) : "memory");
    } else {
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
            ::"r"(smem_u32(dst)), "l"(m), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar)) : "memory");
    }
}

// L2 prefetch of the box tma_load<RANK> would copy with the same coordinates
// (cp.async.bulk.prefetch.tensor: no shared memory, no completion to wait for).
template <int RANK>
__device__ __forceinline__ void tma_prefetch_l2(const CUtensorMap* map, int c0, int c1, int c2, int c3) {
    uint64_t const m = reinterpret_cast<uint64_t>(map);
    if (RANK == 2) {
        asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(m), "r"(c0), "r"(c1)
                     : "memory");
    } else if (RANK == 3) {
        asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(m), "r"(c0), "r"(c1),
                     "r"(c2) : "memory");
    } else {
        asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(m), "r"(c0),
                     "r"(c1), "r"(c2), "r"(c3) : "memory");
    }
}

// ---------------------------------------------------------------------------
// per-cell helpers shared by the stage kernel and the auxiliary kernels
// ---------------------------------------------------------------------------

template <int DIM, class GI>
__device__ __forceinline__ long long padIndex(const GI& I, int gx, int gy, int gz) {
    long long const y = DIM > 1 ? gy + kG : 0;
    long long const z = DIM > 2 ? gz + kG : 0;
    return (z * I.py + y) * I.px + (gx + kG);
}

// The instance geometry the per-cell code indexes with, held in registers for
// a tile: the instance itself lives in global memory, and after each store of
// a cell the compiler would have to load its fields again (a store through a
// T* may alias them).
struct Geo {
    long long plane;
    int px, py;
    int n[3];
    int bc[6];
};

__device__ __forceinline__ Geo geoOf(const DevInst& I) {
    Geo g;
    g.plane = I.plane;
    g.px = I.px;
    g.py = I.py;
#pragma unroll
    for (int k = 0; k < 3; ++k) g.n[k] = I.n[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) g.bc[k] = I.bc[k];
    return g;
}

// Per-tile constants: everything the sweeps and the cell epilogue need from
// the instance, converted once per tile to the arithmetic type (FP64 work per
// cell would run on GB300's narrow FP64 pipe).
template <typename T>
struct TileK {
    fast::Eos<T> fe;      // fast form
    ref::Eos re;          // exact form
    T dtdx[3];            // dt / grid_dx (flux limiter)
    double dtdx_d[3];
    T area[3];            // areaL * invVolume per side
    bool skip[3];         // volume <= 1e-7: the side adds nothing
    bool zero[3];         // area <= 1e-7: zero flux
    T invg1;              // 1 / (gamma - 1)
    T gdx[3];             // grid_dx
    T calpha[4], cbeta[4], cbcur;   // stage coefficients (beta * dt cast to real, as the reference does)
    bool useCur;
};

// Fills the tile constants from the instance (host-converted) and the slot's
// per-step coefficients: loads only, no FP64 arithmetic in the stage kernel.
template <typename T>
__device__ __forceinline__ void makeTileK(TileK<T>& k, const DevInst& I, const DevCtl* c, const StageDev* st,
                                          int slopeLim, int fluxLim, int flux = HC_FLUX_ROE, int hllcMethod = 2,
                                          int recon = HC_RECON_NONE) {
    if constexpr (sizeof(T) == 4) {
        k.fe.gamma = I.f_gamma;
        k.fe.g1 = I.f_g1;
        k.fe.rhoMin = I.f_rhoMin;
        k.fe.PMin = I.f_PMin;
        k.invg1 = I.f_invg1;
    } else {
        k.fe.gamma = I.gamma;
        k.fe.g1 = I.gamma - 1.;
        k.fe.rhoMin = I.rhoMin;
        k.fe.PMin = I.PMin;
        k.invg1 = 1. / (I.gamma - 1.);
    }
    k.fe.fluxLimiter = fluxLim;
    k.fe.slopeLimiter = slopeLim;
    k.fe.entropyFactor = sizeof(T) == 4 ? (T)I.f_entropyFactor : (T)(I.entropyFix ? I.entropyFactor : 0.);
    k.re.entropyFix = I.entropyFix;
    k.re.entropyFactor = I.entropyFactor;
    k.re.gamma = I.gamma;
    k.re.rhoMin = I.rhoMin;
    k.re.PMin = I.PMin;
    k.re.fluxLimiter = fluxLim;
    k.re.slopeLimiter = slopeLim;
    k.re.flux = flux;
    k.re.hllcMethod = hllcMethod;
    k.re.recon = recon;
    k.fe.hllcMethod = hllcMethod;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if constexpr (sizeof(T) == 4) {
            k.area[d] = I.f_area[d];
            k.gdx[d] = I.f_gdx[d];
        } else {
            k.area[d] = I.area[d];
            k.gdx[d] = I.grid_dx[d];
        }
        k.skip[d] = I.skipDeriv[d] != 0;
        k.zero[d] = I.zeroFlux[d] != 0;
        k.dtdx_d[d] = c ? c->dtdx_d[d] : 0.;
        k.dtdx[d] = c ? (sizeof(T) == 4 ? (T)c->dtdx_f[d] : (T)c->dtdx_d[d]) : T(0);
    }
    if (st && c) {
        int const s = st->stage;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            k.calpha[m] = sizeof(T) == 4 ? (T)st->alpha_f[m] : (T)st->alpha[m];
            k.cbeta[m] = sizeof(T) == 4 ? (T)c->cb_f[s][m] : (T)c->cb_d[s][m];
        }
        k.cbcur = sizeof(T) == 4 ? (T)c->cb_f[s][4] : (T)c->cb_d[s][4];
        k.useCur = st->beta_cur != 0.;
    }
}

// constrainU of one cell (global frame, 5 components).
template <typename T, bool EXACT>
__device__ __forceinline__ void constrainCell(T* u, const TileK<T>& K) {
    if constexpr (EXACT) {
        double U[6] = {(double)u[0], (double)u[1], (double)u[2], (double)u[3], (double)u[4], 0.};
        ref::constrain(U, K.re);
        for (int j = 0; j < 5; ++j) u[j] = (T)U[j];
    } else {
        T const rhoMin = K.fe.rhoMin;
        if (u[0] < rhoMin) u[0] = rhoMin;
        T const inv = fast::M<T>::rcp(u[0]);
        T const vx = u[1] * inv, vy = u[2] * inv, vz = u[3] * inv;
        T const m2 = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
        T P = u[0] < rhoMin ? T(0) : K.fe.g1 * (u[4] - T(.5) * m2 * inv);
        if (P < K.fe.PMin) P = K.fe.PMin;
        T const rho = u[0];
        u[1] = vx * rho;
        u[2] = vy * rho;
        u[3] = vz * rho;
        u[4] = rho * (T(.5) * (vx * vx + vy * vy + vz * vz)) + P * K.invg1;
    }
}

// calcDTCell of one cell (global frame).  The minimum over cells is exact in
// any precision; the cross-CTA reduction is done on the FP64 bits.
template <typename T, bool EXACT, int DIM>
__device__ __forceinline__ T dtCell(const T* u, const TileK<T>& K, const DevInst& I) {
    if constexpr (EXACT) {
        double U[6] = {(double)u[0], (double)u[1], (double)u[2], (double)u[3], (double)u[4], 0.};
        return (T)ref::dtCell(U, K.re, DIM, I.grid_dx);
    } else {
        T const rhoMin = K.fe.rhoMin;
        T const inv = fast::M<T>::rcp(u[0]);
        T const m2 = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
        T const P = u[0] < rhoMin ? T(0) : K.fe.g1 * (u[4] - T(.5) * m2 * inv);
        T const Cs = P <= K.fe.PMin ? T(0) : (u[0] < rhoMin ? fast::M<T>::inf() : fast::M<T>::sqrt_(K.fe.gamma * P * inv));
        T dt = fast::M<T>::inf();
#pragma unroll
        for (int side = 0; side < DIM; ++side) {
            T const vn = u[0] < rhoMin ? T(0) : u[1 + side] * inv;
            T a = fast::tmax(fast::M<T>::abs_(vn - Cs), fast::M<T>::abs_(vn + Cs));
            a = fast::tmax(T(1e-9), a);
            dt = fast::tmin(dt, fast::M<T>::div(K.gdx[side], a));
        }
        return dt;
    }
}

// Writes a freshly computed interior cell into every ghost cell that the
// boundary condition copies from it (gridsolver.lua:638-780): periodic wraps,
// mirror reflects with the normal momentum negated, freeflow repeats the edge
// cell.  Corner ghosts are never read by the dimension-split stencil and are
// not written.
template <typename T, int DIM, class GI>
__device__ __forceinline__ void scatterGhosts(const GI& I, T* base, int gx, int gy, int gz, const T* u) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        int const c = d == 0 ? gx : (d == 1 ? gy : gz), N = I.n[d];
        if (c >= 2 && c < N - 2) continue;   // no boundary copies this cell
        // ghost cell at coordinate t along axis d; `neg` negates the normal momentum
        auto put = [&](int t, bool neg) {
            long long const idx = padIndex<DIM>(I, d == 0 ? t : gx, d == 1 ? t : gy, d == 2 ? t : gz);
#pragma unroll
            for (int f = 0; f < 5; ++f) base[f * I.plane + idx] = neg && f == 1 + d ? T(-1) * u[f] : u[f];
        };
        int const lo = I.bc[2 * d], hi = I.bc[2 * d + 1];
        if (lo == HC_BOUNDARY_PERIODIC && c >= N - 2) put(c - N, false);
        if (lo == HC_BOUNDARY_MIRROR && c <= 1) put(-1 - c, true);
        if (lo == HC_BOUNDARY_FREEFLOW && c == 0) { put(-1, false); put(-2, false); }
        if (hi == HC_BOUNDARY_PERIODIC && c <= 1) put(N + c, false);
        if (hi == HC_BOUNDARY_MIRROR && c >= N - 2) put(N + (N - 1 - c), true);
        if (hi == HC_BOUNDARY_FREEFLOW && c == N - 1) { put(N, false); put(N + 1, false); }
    }
}

// ---------------------------------------------------------------------------
// line sweeps
// ---------------------------------------------------------------------------

// deriv - (FR * area - FL * area): calcDerivFromFlux's update of one field
// (fvsolver.cl:37-102).  The exact form keeps the reference's expression.  The
// fast form evaluates deriv + (FL - FR) * area with explicitly rounded
// operations: a sweep's left flux is the previous cell's right flux, so
// unrolled and rolled schedules would otherwise fuse different products into
// FMAs and round differently; this way every schedule gives the same bits.
template <typename T, bool EXACT>
__device__ __forceinline__ T fluxDiff(T deriv, T FL, T FR, T area) {
    if constexpr (EXACT) {
        return deriv - (FR * area - FL * area);
    } else if constexpr (sizeof(T) == 4) {
        return __fmaf_rn(__fsub_rn(FL, FR), area, deriv);
    } else {
        return __fma_rn(__dsub_rn(FL, FR), area, deriv);
    }
}

// Box geometry of a tile configuration.
template <int DIM, int TX, int TY, int TZ>
struct BoxGeom {
    static constexpr int BX = TX + 4;
    static constexpr int BY = DIM > 1 ? TY + 4 : 1;
    static constexpr int BZ = DIM > 2 ? TZ + 4 : 1;
    static constexpr int BOXN = BX * BY * BZ;
    static constexpr int DPX = TX + 1;
    static constexpr int DN = DPX * (DIM > 1 ? TY : 1) * (DIM > 2 ? TZ : 1);
};

// Sweeps one segment of L cells along AXIS.  `base` is the box index of the
// segment's first cell.  emit(k, FL, FR) receives, for cell k of the segment,
// its left and right face fluxes in the global frame (5 components).
// UNR: unroll factor of the sliding-window loop (0: fully unrolled).  Full
// unrolling removes the window copies; partial unrolling keeps the code
// footprint inside the instruction cache.
template <typename T, int AXIS, int STRIDE, int BOXN, int L, bool EXACT, int PLM, bool LIM, int SLOPE, int UNR, class Emit>
__device__ __forceinline__ void sweepSegment(const T* box, int base, const TileK<T>& K, Emit&& emit) {
    // SLOPE >= 0 fixes the slope limiter at compile time; -1 dispatches at run time
    int const slopeLim = SLOPE >= 0 ? SLOPE : K.fe.slopeLimiter;
    if constexpr (EXACT) {
        ref::Eos const& e = K.re;
        double const dt_dx = K.dtdx_d[AXIS];
        auto load = [&](int k, double* U) {
#pragma unroll
            for (int f = 0; f < 5; ++f) U[f] = (double)box[f * BOXN + base + k * STRIDE];
            U[5] = 0.;
        };
        double Fprev[6], F[6];
        bool const zero = K.zero[AXIS];
        auto flux = [&](double* out, const double* UL, const double* UR, const ref::Iface& C,
                        const ref::Iface* IL, const ref::Iface* IR) {
            if (zero) { for (int j = 0; j < 6; ++j) out[j] = 0.; return; }
            if (e.flux == HC_FLUX_RUSANOV) {
                ref::rusanovFlux(out, e, UL, UR, AXIS);
            } else if (e.flux == HC_FLUX_HLL || e.flux == HC_FLUX_HLLC) {
                // a NaN wave bound assigns nothing in the reference (its flux
                // buffer keeps stale values); this form has no flux buffer
                bool const set = e.flux == HC_FLUX_HLL ? ref::hllFlux(out, e, UL, UR, AXIS, C.eig)
                                                       : ref::hllcFlux(out, e, UL, UR, AXIS, C.eig);
                if (!set)
                    for (int j = 0; j < 6; ++j) out[j] = __longlong_as_double(0x7ff8000000000000ll);
            } else {
                ref::roeFlux(out, e, UL, UR, C, IL, IR, AXIS, LIM, dt_dx);
            }
        };
        if constexpr (PLM != 0) {
            double Um[6], U0[6], Up[6], prevR[6], fL[6], fR[6];
            load(-2, Um);
            load(-1, U0);
            for (int k = -1; k <= L; ++k) {
                load(k + 1, Up);
                ref::plmAny(fL, fR, e, Um, U0, Up, AXIS);
                if (k >= 0) {
                    ref::Iface C;
                    ref::makeIface(C, e, prevR, fL, AXIS);
                    flux(F, prevR, fL, C, &C, &C);
                    if (k >= 1) emit(k - 1, Fprev, F);
                    for (int j = 0; j < 6; ++j) Fprev[j] = F[j];
                }
                for (int j = 0; j < 6; ++j) { prevR[j] = fR[j]; Um[j] = U0[j]; U0[j] = Up[j]; }
            }
        } else if constexpr (LIM) {
            double Ua[6], Ub[6], Uc[6], Ud[6];
            ref::Iface IL, IC, IR;
            load(-2, Ua);
            load(-1, Ub);
            load(0, Uc);
            ref::makeIface(IL, e, Ua, Ub, AXIS);
            ref::makeIface(IC, e, Ub, Uc, AXIS);
            for (int k = 0; k <= L; ++k) {
                load(k + 1, Ud);
                ref::makeIface(IR, e, Uc, Ud, AXIS);
                flux(F, Ub, Uc, IC, &IL, &IR);
                if (k >= 1) emit(k - 1, Fprev, F);
                for (int j = 0; j < 6; ++j) { Fprev[j] = F[j]; Ub[j] = Uc[j]; Uc[j] = Ud[j]; }
                IL = IC;
                IC = IR;
            }
        } else {
            double Ua[6], Ub[6];
            load(-1, Ua);
            for (int k = 0; k <= L; ++k) {
                load(k, Ub);
                ref::Iface C;
                ref::makeIface(C, e, Ua, Ub, AXIS);
                flux(F, Ua, Ub, C, &C, &C);
                if (k >= 1) emit(k - 1, Fprev, F);
                for (int j = 0; j < 6; ++j) { Fprev[j] = F[j]; Ua[j] = Ub[j]; }
            }
        }
    } else {
        // the fast form with the flux limiter (the others run sweepLanes)
        static_assert(LIM && PLM == 0, "the fast form sweeps here only with the flux limiter");
        using C5 = fast::C5<T>;
        fast::Eos<T> const& e = K.fe;
        T const dt_dx = K.dtdx[AXIS];
        constexpr int A1 = 1 + AXIS, A2 = 1 + (AXIS + 1) % 3, A3 = 1 + (AXIS + 2) % 3;
        // loads in the interface frame (rho, m_n, m_t1, m_t2, E)
        auto load = [&](int k, C5& U) {
            int const i = base + k * STRIDE;
            U.u[0] = box[0 * BOXN + i];
            U.u[1] = box[A1 * BOXN + i];
            U.u[2] = box[A2 * BOXN + i];
            U.u[3] = box[A3 * BOXN + i];
            U.u[4] = box[4 * BOXN + i];
        };
        bool const zero = K.zero[AXIS];
        T Fprev[5], F[5];
        C5 Ua, Ub, Uc, Ud;
        fast::IfaceF<T> IL, IC, IR;
        load(-2, Ua);
        load(-1, Ub);
        load(0, Uc);
        fast::makeIface(IL, e, Ua, Ub);
        fast::makeIface(IC, e, Ub, Uc);
#pragma unroll 1
        for (int k = 0; k <= L; ++k) {
            load(k + 1, Ud);
            fast::makeIface(IR, e, Uc, Ud);
            T Fr[5];
            fast::roeLimited<T>(Fr, e, Ub, Uc, IC, IL, IR, dt_dx);
            if (zero) for (int j = 0; j < 5; ++j) Fr[j] = T(0);
            F[0] = Fr[0];
            F[A1] = Fr[1];
            F[A2] = Fr[2];
            F[A3] = Fr[3];
            F[4] = Fr[4];
            if (k >= 1) emit(k - 1, Fprev, F);
#pragma unroll
            for (int j = 0; j < 5; ++j) Fprev[j] = F[j];
            Ub = Uc;
            Uc = Ud;
            IL = IC;
            IC = IR;
        }
    }
}

// Sweeps one segment of L cells along AXIS on nlanes<V>() neighbouring lines
// at once (fast form, no flux limiter): lane l's line starts at box index
// base + l * LSTRIDE.  emit(k, FL, FR) receives, for cell k of the segment,
// the left and right face fluxes of every lane in the global frame.
template <typename V, int AXIS, int STRIDE, int LSTRIDE, int BOXN, int L, int PLM, int SLOPE, int UNR, int FLUX,
          class Emit>
__device__ __forceinline__ void sweepLanes(const float* box, int base, const lanes::Eos& e, int slopeLim, bool zero,
                                           Emit&& emit) {
    using C5 = lanes::C5<V>;
    constexpr int A1 = 1 + AXIS, A2 = 1 + (AXIS + 1) % 3, A3 = 1 + (AXIS + 2) % 3;
    constexpr int NL = lanes::nlanes<V>();
    auto ld = [&](int f, int i) -> V {
        V v;
        if constexpr (NL == 1) {
            v = box[f * BOXN + i];
        } else if constexpr (LSTRIDE == 1) {
            v = *reinterpret_cast<const float2*>(box + f * BOXN + i);   // neighbouring columns: one 8-byte load
        } else {
            v = make_float2(box[f * BOXN + i], box[f * BOXN + i + LSTRIDE]);
        }
        return v;
    };
    // loads in the interface frame (rho, m_n, m_t1, m_t2, E)
    auto load = [&](int k, C5& U) {
        int const i = base + k * STRIDE;
        U.u[0] = ld(0, i);
        U.u[1] = ld(A1, i);
        U.u[2] = ld(A2, i);
        U.u[3] = ld(A3, i);
        U.u[4] = ld(4, i);
    };
    V F[5], Fprev[5];
    auto flux = [&](const C5& UL, const C5& UR) {
        V Fr[5];
        if constexpr (FLUX == HC_FLUX_HLL) lanes::hll<V>(Fr, e, UL, UR);
        else if constexpr (FLUX == HC_FLUX_HLLC) lanes::hllc<V>(Fr, e, UL, UR);
        else if constexpr (FLUX == HC_FLUX_RUSANOV) lanes::rusanov<V>(Fr, e, UL, UR);
        else lanes::roe<V>(Fr, e, UL, UR);
        if (zero) for (int j = 0; j < 5; ++j) Fr[j] = lanes::splat<V>(0.f);
        F[0] = Fr[0];
        F[A1] = Fr[1];
        F[A2] = Fr[2];
        F[A3] = Fr[3];
        F[4] = Fr[4];
    };
    if constexpr (PLM == HC_RECON_PLM_CONS) {
        C5 Um, U0, Up, prevR, fL, fR;
        V dL[5];
        load(-2, Um);
        load(-1, U0);
#pragma unroll
        for (int j = 0; j < 5; ++j) dL[j] = lanes::sub(U0.u[j], Um.u[j]);
#pragma unroll (UNR == 0 ? L + 2 : UNR)
        for (int k = -1; k <= L; ++k) {
            load(k + 1, Up);
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                V const dR = lanes::sub(Up.u[j], U0.u[j]);
                V const h = lanes::halfSlope<SLOPE>(dL[j], dR, slopeLim);
                fL.u[j] = lanes::sub(U0.u[j], h);
                fR.u[j] = lanes::add(U0.u[j], h);
                dL[j] = dR;
            }
            if (k >= 0) {
                flux(prevR, fL);
                if (k >= 1) emit(k - 1, Fprev, F);
#pragma unroll
                for (int j = 0; j < 5; ++j) Fprev[j] = F[j];
            }
            prevR = fR;
            Um = U0;
            U0 = Up;
        }
    } else if constexpr (PLM != 0) {
        // "plm prim" / "plm athena", or (PLM < 0) the reconstruction the
        // scheme names, chosen at run time; the window keeps each cell's
        // primitives next to its conserved state
        C5 Um, U0, Up, prevR, fL, fR;
        V Wm[5], W0[5], Wp[5];
        load(-2, Um);
        lanes::primOf(Wm, e, Um);
        load(-1, U0);
        lanes::primOf(W0, e, U0);
        int const rc = PLM > 0 ? PLM : e.recon;
#pragma unroll 1
        for (int k = -1; k <= L; ++k) {
            load(k + 1, Up);
            lanes::primOf(Wp, e, Up);
            if (rc == HC_RECON_PLM_ATHENA) {
                lanes::plmAthena<V>(fL, fR, e, U0, Wm, W0, Wp);
            } else if (rc == HC_RECON_PLM_PRIM) {
                lanes::plmPrim<V>(fL, fR, e, Wm, W0, Wp, slopeLim);
            } else {
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    V const h = lanes::halfSlope<SLOPE>(lanes::sub(U0.u[j], Um.u[j]), lanes::sub(Up.u[j], U0.u[j]),
                                                        slopeLim);
                    fL.u[j] = lanes::sub(U0.u[j], h);
                    fR.u[j] = lanes::add(U0.u[j], h);
                }
            }
            if (k >= 0) {
                flux(prevR, fL);
                if (k >= 1) emit(k - 1, Fprev, F);
#pragma unroll
                for (int j = 0; j < 5; ++j) Fprev[j] = F[j];
            }
            prevR = fR;
            Um = U0;
            U0 = Up;
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                Wm[j] = W0[j];
                W0[j] = Wp[j];
            }
        }
    } else {
        C5 Ua, Ub;
        load(-1, Ua);
#pragma unroll (UNR == 0 ? L + 1 : UNR)
        for (int k = 0; k <= L; ++k) {
            load(k, Ub);
            flux(Ua, Ub);
            if (k >= 1) emit(k - 1, Fprev, F);
#pragma unroll
            for (int j = 0; j < 5; ++j) Fprev[j] = F[j];
            Ua = Ub;
        }
    }
}

__device__ __forceinline__ double laneOf(double v, int) { return v; }
__device__ __forceinline__ float laneOf(float v, int) { return v; }
__device__ __forceinline__ float laneOf(float2 v, int k) { return k ? v.y : v.x; }

// One segment sweep: the FP32 fast form without a flux limiter runs the
// lane-generic arithmetic (LANES lines at once); the exact form and the
// flux-limited fast form run sweepSegment (one line).
template <typename T, int AXIS, int STRIDE, int LSTRIDE, int BOXN, int L, bool EXACT, int PLM, bool LIM, int SLOPE,
          int UNR, int LANES, int FLUX, class Emit>
__device__ __forceinline__ void sweepAny(const T* box, int base, const TileK<T>& K, Emit&& emit) {
    if constexpr (!EXACT && !LIM && sizeof(T) == 4) {
        using V = typename std::conditional<LANES == 2, float2, float>::type;
        lanes::Eos const e{K.fe.gamma, K.fe.g1, K.fe.rhoMin, K.fe.PMin, K.fe.hllcMethod, K.invg1, K.re.recon,
                             (float)K.fe.entropyFactor};
        sweepLanes<V, AXIS, STRIDE, LSTRIDE, BOXN, L, PLM, SLOPE, UNR, FLUX>(
            box, base, e, SLOPE >= 0 ? SLOPE : K.fe.slopeLimiter, K.zero[AXIS], emit);
    } else {
        static_assert(LANES == 1, "two-lane sweeps need the FP32 fast form without a flux limiter");
        sweepSegment<T, AXIS, STRIDE, BOXN, L, EXACT, PLM, LIM, SLOPE, UNR>(box, base, K, emit);
    }
}

// ---------------------------------------------------------------------------
// the stage kernel
// ---------------------------------------------------------------------------

template <typename T, int DIM, int TX, int TY, int TZ, int L, int NT>
struct StageCfg {
    using G = BoxGeom<DIM, TX, TY, TZ>;
    static constexpr size_t kBarOff = (((size_t)(5 * G::BOXN + 5 * G::DN) * sizeof(T)) + 15) / 16 * 16;
    static constexpr size_t SMEM = kBarOff + 16;
    static constexpr unsigned BYTES = (unsigned)(5 * G::BOXN * sizeof(T));
    static_assert(G::BX <= 256 && G::BY <= 256 && G::BZ <= 256, "TMA box extent");
    static_assert((G::BX * sizeof(T)) % 16 == 0, "TMA box rows must be a multiple of 16 bytes");
    static_assert(TX % L == 0 && (DIM < 2 || TY % L == 0) && (DIM < 3 || TZ % L == 0), "segments tile the box");
};

constexpr unsigned kSpinLimit = 1u << 22;

// Resident CTAs per SM that a configuration's shared memory allows (228 KB per
// SM, 1 KB reserved per CTA) and its thread count allows (2048 per SM).  The
// stage kernel declares it as its minimum, so the compiler may use every
// register that occupancy leaves (65536 / (CTAs x threads)) instead of
// spilling to reach an occupancy the shared memory rules out anyway.
constexpr int residentCtas(int nt, size_t smem) {
    int const bySmem = (int)((size_t)228 * 1024 / (smem + 1024));
    int const byThreads = 2048 / nt;
    int const o = bySmem < byThreads ? bySmem : byThreads;
    return o > 32 ? 32 : (o < 1 ? 1 : o);
}

// FLUX: the interface flux of the fast form (HC_FLUX_*); the exact form
// reads it from the launch arguments.
template <typename T, int DIM, int TX, int TY, int TZ, int L, int NT, bool EXACT, int PLM, bool LIM, int SLOPE, int UNR,
          int OCC, int LANES, int FLUX>
__global__ void __launch_bounds__(NT, OCC) k_stage(const __grid_constant__ StageArgs a, int slopeLim, int fluxLim) {
    static_assert(LANES == 1 || (DIM >= 2 && TX % 2 == 0 && TY % 2 == 0), "two-lane sweeps pair rows and columns");
    using Cfg = StageCfg<T, DIM, TX, TY, TZ, L, NT>;
    using G = typename Cfg::G;
    extern __shared__ __align__(128) unsigned char smem[];
    T* box = reinterpret_cast<T*>(smem);
    T* D = box + 5 * G::BOXN;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Cfg::kBarOff);
    int const tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    __syncthreads();

    int const nitems = *a.nitems;
    unsigned phase = 0;
    const StageDev& st = a.st;

    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        int4 const it = a.items[item];
        const DevInst& I = a.inst[it.x];
        DevCtl* ctl = a.ctl + it.x;
        if (!ctl->stepping) continue;
        int const x0 = it.y * TX, y0 = it.z * TY, z0 = it.w * TZ;
        int const rot = ctl->rot;
        int const inBuf = slotBuf(st.in_buf, rot, a.rot_buf);

        if (tid == 0) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, Cfg::BYTES);
            const CUtensorMap* map = a.tmaps + (size_t)it.x * kMaxBufs + inBuf;
            if (DIM == 1) tma_load<2>(box, map, x0, 0, 0, 0, bar);
            else if (DIM == 2) tma_load<3>(box, map, x0, y0, 0, 0, bar);
            else tma_load<4>(box, map, x0, y0, z0, 0, bar);
            // the first other RK state this tile's cells combine (read from
            // global memory by the epilogue) into L2 while the sweeps run; one
            // tensor prefetch per state would put up to three back to back
            // (RK4-TVD), a pattern under which an earlier kernel faulted
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (m >= st.n_alpha) break;
                int const b = slotBuf(st.alpha_buf[m], rot, a.rot_buf);
                if (b == inBuf) continue;
                const CUtensorMap* amap = a.tmaps + (size_t)it.x * kMaxBufs + b;
                if (DIM == 1) tma_prefetch_l2<2>(amap, x0, 0, 0, 0);
                else if (DIM == 2) tma_prefetch_l2<3>(amap, x0, y0, 0, 0);
                else tma_prefetch_l2<4>(amap, x0, y0, z0, 0);
                break;
            }
            // the box of this CTA's next item into L2 while this one is computed
            int const next = item + (int)gridDim.x;
            if (next < nitems) {
                int4 const nt = a.items[next];
                const DevCtl* nc = a.ctl + nt.x;
                if (nc->stepping) {
                    const CUtensorMap* nmap = a.tmaps + (size_t)nt.x * kMaxBufs + slotBuf(st.in_buf, nc->rot, a.rot_buf);
                    if (DIM == 1) tma_prefetch_l2<2>(nmap, nt.y * TX, 0, 0, 0);
                    else if (DIM == 2) tma_prefetch_l2<3>(nmap, nt.y * TX, nt.z * TY, 0, 0);
                    else tma_prefetch_l2<4>(nmap, nt.y * TX, nt.z * TY, nt.w * TZ, 0);
                }
            }
        }
        // the tile's constants (loads; no FP64 arithmetic) while the tile streams in
        TileK<T> K;
        makeTileK<T>(K, I, ctl, &st, slopeLim, fluxLim, a.flux, a.hllcMethod, a.recon);
        if (a.force_timeout || !mbar_wait_bounded(bar, phase, kSpinLimit)) {
            // the copy did not complete: record it, give the copy a second
            // bounded chance to land before the CTA releases its smem, stop
            if (tid == 0) { atomicOr(a.err, DEV_TIMEOUT); atomicOr(&ctl->status, DEV_TIMEOUT); }
            mbar_wait_bounded(bar, phase, kSpinLimit);
            return;
        }
        phase ^= 1u;

        int const nx = I.n[0], ny = I.n[1], nz = I.n[2];

        // ---- all axes but the last: flux differences into D ----------------
        // (LANES = 2: each thread sweeps two neighbouring lines in lockstep)
        if constexpr (DIM >= 2) {
#pragma unroll 1
            for (int axis = 0; axis < DIM - 1; ++axis) {
                if (axis == 0) {
                    // lines along x, indexed by (cy, cz); lanes are neighbouring rows
                    constexpr int nlines = TY / LANES * (DIM > 2 ? TZ : 1);
                    constexpr int nseg = TX / L;
                    T const ar = K.area[0];
                    bool const skip = K.skip[0];
                    for (int t = tid; t < nlines * nseg; t += NT) {
                        int const line = t % nlines, seg = t / nlines;
                        int const cy = (line % (TY / LANES)) * LANES, cz = line / (TY / LANES);
                        int const cx0 = seg * L;
                        if (x0 + cx0 >= nx || y0 + cy >= ny || z0 + cz >= nz) continue;
                        int const base = ((cz + (DIM > 2 ? 2 : 0)) * G::BY + (cy + 2)) * G::BX + (cx0 + 2);
                        T* Dl = D + (cz * TY + cy) * G::DPX + cx0;
                        sweepAny<T, 0, 1, G::BX, G::BOXN, L, EXACT, PLM, LIM, SLOPE, UNR, LANES, FLUX>(box, base, K,
                            [&](int k, const auto* FL, const auto* FR) {
#pragma unroll
                                for (int l = 0; l < LANES; ++l)
#pragma unroll
                                    for (int f = 0; f < 5; ++f) {
                                        T d = T(0);
                                        if (!skip) d = fluxDiff<T, EXACT>(T(0), T(laneOf(FL[f], l)), T(laneOf(FR[f], l)), ar);
                                        Dl[f * G::DN + l * G::DPX + k] = d;
                                    }
                            });
                    }
                } else if constexpr (DIM == 3) {
                    // axis 1 of a 3D tile: lines along y, indexed by (cx, cz); lanes are neighbouring columns
                    constexpr int nlines = TX / LANES * TZ;
                    constexpr int nseg = TY / L;
                    T const ar = K.area[1];
                    bool const skip = K.skip[1];
                    for (int t = tid; t < nlines * nseg; t += NT) {
                        int const cx = (t % (TX / LANES)) * LANES, rest = t / (TX / LANES);
                        int const cz = rest % TZ, seg = rest / TZ;
                        int const cy0 = seg * L;
                        if (x0 + cx >= nx || y0 + cy0 >= ny || z0 + cz >= nz) continue;
                        int const base = ((cz + 2) * G::BY + (cy0 + 2)) * G::BX + (cx + 2);
                        T* Dl = D + (cz * TY + cy0) * G::DPX + cx;
                        sweepAny<T, 1, G::BX, 1, G::BOXN, L, EXACT, PLM, LIM, SLOPE, UNR, LANES, FLUX>(box, base, K,
                            [&](int k, const auto* FL, const auto* FR) {
#pragma unroll
                                for (int l = 0; l < LANES; ++l)
#pragma unroll
                                    for (int f = 0; f < 5; ++f) {
                                        T& d = Dl[f * G::DN + k * G::DPX + l];
                                        if (!skip) d = fluxDiff<T, EXACT>(d, T(laneOf(FL[f], l)), T(laneOf(FR[f], l)), ar);
                                    }
                            });
                    }
                }
                __syncthreads();
            }
        }

        // ---- last axis: sweep into D, then finish each of the segment's cells
        constexpr int AX = DIM - 1;
        constexpr int TA = AX == 0 ? TX : (AX == 1 ? TY : TZ);
        constexpr int nlines = (TX * TY * TZ) / TA / (DIM < 2 ? TY : 1) / (DIM < 3 ? TZ : 1) / LANES;
        constexpr int nseg = TA / L;
        constexpr int STRIDE_AX = AX == 0 ? 1 : (AX == 1 ? G::BX : G::BX * G::BY);
        constexpr int DSTRIDE_AX = AX == 0 ? 1 : (AX == 1 ? G::DPX : G::DPX * TY);

        T const cbcur = K.cbcur;
        bool const useCur = K.useCur;
        T* out = reinterpret_cast<T*>(I.buf[slotBuf(st.out_buf, rot, a.rot_buf)]);
        T* dstore = st.store_deriv >= 0 ? reinterpret_cast<T*>(I.dbuf[st.store_deriv]) : nullptr;
        // The geometry and source buffers the cells of a segment use.  With
        // registers to spare (the launch bounds leave >= 96 a thread) they are
        // loaded into registers once per segment, after its sweep; otherwise
        // the cell code reads them from the instance (holding them would make
        // the register-tight schedules spill).
        constexpr bool HOIST = 65536 / (NT * (OCC > 0 ? OCC : 1)) >= 96;
        Geo geo;
        const T* asrc[4];
        bool afromBox[4];
        const T* bsrc[4];
        auto loadEpilogue = [&]() {
            if constexpr (HOIST) {
                geo = geoOf(I);
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    int const b = m < st.n_alpha ? slotBuf(st.alpha_buf[m], rot, a.rot_buf) : inBuf;
                    afromBox[m] = b == inBuf;
                    asrc[m] = reinterpret_cast<const T*>(I.buf[b]);
                    bsrc[m] = m < st.n_beta ? reinterpret_cast<const T*>(I.dbuf[st.beta_buf[m]]) : nullptr;
                }
            }
        };
        auto const& gi = [&]() -> decltype(auto) {
            if constexpr (HOIST) return (geo);
            else return (I);
        }();
        auto fromBoxA = [&](int m) -> bool {
            if constexpr (HOIST) return afromBox[m];
            else return slotBuf(st.alpha_buf[m], rot, a.rot_buf) == inBuf;
        };
        auto srcA = [&](int m) -> const T* {
            if constexpr (HOIST) return asrc[m];
            else return reinterpret_cast<const T*>(I.buf[slotBuf(st.alpha_buf[m], rot, a.rot_buf)]);
        };
        auto srcB = [&](int m) -> const T* {
            if constexpr (HOIST) return bsrc[m];
            else return reinterpret_cast<const T*>(I.dbuf[st.beta_buf[m]]);
        };
        T const arF = K.area[AX];
        bool const skipF = K.skip[AX];
        T dtmin = fast::M<T>::inf();
        bool bad = false;

        // the cell at global (gx, gy, gz), box index bi, accumulator Dc:
        // Runge-Kutta combination, constrainU, store, ghost copies, stored
        // derivative, CFL dt
        auto finishCell = [&](int gx, int gy, int gz, int bi, const T* Dc) {
            long long const idx = padIndex<DIM>(gi, gx, gy, gz);
            T u[5], deriv[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                deriv[f] = Dc[f * G::DN];
                u[f] = T(0);
            }
            // u = sum alpha_k u^(k) + sum (beta_k dt) L(u^(k)) + (beta_cur dt) deriv
            // (loops unrolled to their bound so the coefficients stay in registers)
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (m >= st.n_alpha) break;
                if (fromBoxA(m)) {
#pragma unroll
                    for (int f = 0; f < 5; ++f) u[f] = u[f] + box[f * G::BOXN + bi] * K.calpha[m];
                } else {
                    const T* src = srcA(m);
#pragma unroll
                    for (int f = 0; f < 5; ++f) u[f] = u[f] + src[f * gi.plane + idx] * K.calpha[m];
                }
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (m >= st.n_beta) break;
                const T* src = srcB(m);
#pragma unroll
                for (int f = 0; f < 5; ++f) u[f] = u[f] + src[f * gi.plane + idx] * K.cbeta[m];
            }
            if (useCur) {
#pragma unroll
                for (int f = 0; f < 5; ++f) u[f] = u[f] + deriv[f] * cbcur;
            }
            constrainCell<T, EXACT>(u, K);
#pragma unroll
            for (int f = 0; f < 5; ++f) out[f * gi.plane + idx] = u[f];
            // after constrainU a non-finite momentum shows in ETotal
            bad |= !fast::M<T>::finite_(u[0] + u[4]);
            scatterGhosts<T, DIM>(gi, out, gx, gy, gz, u);
            if (dstore) {
#pragma unroll
                for (int f = 0; f < 5; ++f) dstore[f * gi.plane + idx] = deriv[f];
            }
            if (st.last) dtmin = fast::tmin(dtmin, dtCell<T, EXACT, DIM>(u, K, I));
        };

        // the fast form's epilogue, written with the lane operations: V = float
        // finishes the cell (gx, gy, gz); V = float2 finishes it and its +x
        // neighbour with packed arithmetic and 8-byte loads and stores, or
        // only the first when `second` is false (the neighbour is a ghost or
        // padding cell: loaded and computed, never stored)
        auto finishFast = [&](auto vtag, int gx, int gy, int gz, int bi, const T* Dc, bool second) {
            using V = decltype(vtag);
            constexpr int NL = lanes::nlanes<V>();
            long long const idx = padIndex<DIM>(gi, gx, gy, gz);
            auto ld = [&](const T* p) -> V {
                if constexpr (NL == 1) return *p;
                else return *reinterpret_cast<const float2*>(p);
            };
            auto st_ = [&](T* p, V v) {
                if constexpr (NL == 1) *p = v;
                else if (second) *reinterpret_cast<float2*>(p) = v;
                else *p = lanes::lane(v, 0);
            };
            lanes::Eos const le{K.fe.gamma, K.fe.g1, K.fe.rhoMin, K.fe.PMin, K.fe.hllcMethod, K.invg1, K.re.recon,
                             (float)K.fe.entropyFactor};
            V u[5], deriv[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                if constexpr (NL == 1) deriv[f] = Dc[f * G::DN];
                else deriv[f] = make_float2(Dc[f * G::DN], Dc[f * G::DN + 1]);
                u[f] = lanes::splat<V>(0.f);
            }
            // sum alpha_k u^(k) as p + sum_{k < last} alpha_k (u^(k) - p), p the
            // last alpha term: every integrator's alpha row sums to 1, and in
            // this form the weights sum to exactly 1 whatever the FP32 rounding
            // of the alphas (summed directly, RK3-TVD's 1/3 and 2/3 rounded to
            // FP32 add 3e-8 of every conserved quantity per step)
            auto ldAlpha = [&](int m, V* v) {
                if (fromBoxA(m)) {
#pragma unroll
                    for (int f = 0; f < 5; ++f) v[f] = ld(box + f * G::BOXN + bi);
                } else {
                    const T* src = srcA(m);
#pragma unroll
                    for (int f = 0; f < 5; ++f) v[f] = ld(src + f * gi.plane + idx);
                }
            };
            int const last = st.n_alpha - 1;
            V p[5];
#pragma unroll
            for (int m = 0; m < 4; ++m)
                if (m == last) ldAlpha(m, p);
#pragma unroll
            for (int f = 0; f < 5; ++f) u[f] = p[f];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                if (m >= last) break;
                V const c = lanes::splat<V>(K.calpha[m]);
                V w[5];
                ldAlpha(m, w);
#pragma unroll
                for (int f = 0; f < 5; ++f) u[f] = lanes::fma(lanes::sub(w[f], p[f]), c, u[f]);
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (m >= st.n_beta) break;
                const T* src = srcB(m);
                V const c = lanes::splat<V>(K.cbeta[m]);
#pragma unroll
                for (int f = 0; f < 5; ++f) u[f] = lanes::fma(ld(src + f * gi.plane + idx), c, u[f]);
            }
            if (useCur) {
                V const c = lanes::splat<V>(cbcur);
#pragma unroll
                for (int f = 0; f < 5; ++f) u[f] = lanes::fma(deriv[f], c, u[f]);
            }
            lanes::constrain<V>(u, le, K.invg1);
#pragma unroll
            for (int f = 0; f < 5; ++f) st_(out + f * gi.plane + idx, u[f]);
            if (dstore) {
#pragma unroll
                for (int f = 0; f < 5; ++f) st_(dstore + f * gi.plane + idx, deriv[f]);
            }
            V dtv;
            if (st.last) dtv = lanes::dtCell<V, DIM>(u, le, K.gdx);
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                if (l > 0 && !second) break;
                T uu[5];
#pragma unroll
                for (int f = 0; f < 5; ++f) uu[f] = lanes::lane(u[f], l);
                // after constrainU a non-finite momentum shows in ETotal
                bad |= !fast::M<T>::finite_(uu[0] + uu[4]);
                scatterGhosts<T, DIM>(gi, out, gx + l, gy, gz, uu);
                if (st.last) dtmin = fast::tmin(dtmin, lanes::lane(dtv, l));
            }
        };

        for (int t = tid; t < nlines * nseg; t += NT) {
            int cx, cy, cz, seg;
            if (DIM == 1) { cx = 0; cy = 0; cz = 0; seg = t; }
            else if (DIM == 2) { cx = (t % (TX / LANES)) * LANES; seg = t / (TX / LANES); cy = 0; cz = 0; }
            else { cx = (t % (TX / LANES)) * LANES; cy = (t / (TX / LANES)) % TY; seg = t / (TX / LANES * TY); cz = 0; }
            int c0[3] = {cx, cy, cz};
            c0[AX] = seg * L;
            int const gx0 = x0 + c0[0], gy0 = y0 + c0[1], gz0 = z0 + c0[2];
            if (gx0 >= nx || gy0 >= ny || gz0 >= nz) continue;
            int const base = ((c0[2] + (DIM > 2 ? 2 : 0)) * G::BY + (c0[1] + (DIM > 1 ? 2 : 0))) * G::BX + (c0[0] + 2);
            T* Dl = D + (c0[2] * TY + c0[1]) * G::DPX + c0[0];
            sweepAny<T, AX, STRIDE_AX, 1, G::BOXN, L, EXACT, PLM, LIM, SLOPE, UNR, LANES, FLUX>(box, base, K,
                [&](int k, const auto* FL, const auto* FR) {
#pragma unroll
                    for (int l = 0; l < LANES; ++l)
#pragma unroll
                        for (int f = 0; f < 5; ++f) {
                            T& d = Dl[f * G::DN + k * DSTRIDE_AX + l];
                            T dv = DIM > 1 ? d : T(0);
                            if (!skipF) dv = fluxDiff<T, EXACT>(dv, T(laneOf(FL[f], l)), T(laneOf(FR[f], l)), arF);
                            d = dv;
                        }
                });
            int const gA0 = AX == 0 ? gx0 : (AX == 1 ? gy0 : gz0);
            int const nA = AX == 0 ? nx : (AX == 1 ? ny : nz);
            int const kmax = nA - gA0 < L ? nA - gA0 : L;
            loadEpilogue();
            if constexpr (EXACT) {
#pragma unroll 1
                for (int k = 0; k < kmax; ++k) {
                    int g[3] = {gx0, gy0, gz0};
                    g[AX] += k;
                    finishCell(g[0], g[1], g[2], base + k * STRIDE_AX, Dl + k * DSTRIDE_AX);
                }
            } else {
                // LANES = 2: the line pair; the second line may lie beyond the grid
                bool const pair = LANES == 2 && gx0 + 1 < nx;
#pragma unroll 1
                for (int k = 0; k < kmax; ++k) {
                    int g[3] = {gx0, gy0, gz0};
                    g[AX] += k;
                    if constexpr (LANES == 2)
                        finishFast(float2{}, g[0], g[1], g[2], base + k * STRIDE_AX, Dl + k * DSTRIDE_AX, pair);
                    else
                        finishFast(T{}, g[0], g[1], g[2], base + k * STRIDE_AX, Dl + k * DSTRIDE_AX, true);
                }
            }
        }
        // one FP64 atomicMin per warp for the next step's CFL dt
        if (st.last) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dtmin = fast::tmin(dtmin, __shfl_xor_sync(0xffffffffu, dtmin, o));
            double const m = (double)dtmin;
            if ((tid & 31) == 0 && m < __longlong_as_double((long long)kInfBits))
                atomicMin(&ctl->dtmin[ctl->par ^ 1], (unsigned long long)__double_as_longlong(m));
        }
        if (__any_sync(0xffffffffu, bad) && (tid & 31) == 0) atomicOr(&ctl->status, DEV_NONFINITE);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// auxiliary kernels (per slot)
// ---------------------------------------------------------------------------

// Finishes a pending step (t += dt) and begins the next one for every slot:
// the App's exit test (t >= t_end, before stepping), then dt = cfl * min.
__global__ void k_begin(DevCtl* ctl, const DevInst* inst, int nslots, int begin, int rotates, BetaTable bt, int* work);

template <typename T, int DIM>
__global__ void k_fill_ghosts(const DevInst* inst, int slot, int buf) {
    const DevInst& I = inst[slot];
    T* base = reinterpret_cast<T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
        bool edge = false;
        int g[3] = {gx, gy, gz};
        for (int d = 0; d < DIM; ++d) edge |= g[d] < 2 || g[d] >= I.n[d] - 2;
        if (!edge) continue;
        long long const idx = padIndex<DIM>(I, gx, gy, gz);
        T u[5];
        for (int f = 0; f < 5; ++f) u[f] = base[f * I.plane + idx];
        scatterGhosts<T, DIM>(I, base, gx, gy, gz, u);
    }
}

// The fixed boundaries (gridsolver.lua:746-765) of one instance: the two
// ghost layers of every HC_BOUNDARY_FIXED side take the side's constant state
// in each of the first `nbufs` state buffers, on the lines through the
// interior (corner ghosts are never read).  No stage writes these ghosts, so
// this runs once when the instance is set up.
template <typename T, int DIM>
__global__ void k_fixed_ghosts(const DevInst* inst, int slot, int nbufs) {
    const DevInst& I = inst[slot];
    long long const stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 1
    for (int d = 0; d < DIM; ++d) {
        int const o1 = (d + 1) % 3, o2 = (d + 2) % 3;
        long long const nface = (long long)I.n[o1] * I.n[o2];
#pragma unroll 1
        for (int mm = 0; mm < 2; ++mm) {
            if (I.bc[2 * d + mm] != HC_BOUNDARY_FIXED) continue;
            const double* const v = I.fixedCons[2 * d + mm];
            for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nface * 2 * nbufs; k += stride) {
                long long const cell = k % nface;
                int const j = (int)((k / nface) % 2), b = (int)(k / (2 * nface));
                int c[3];
                c[o1] = (int)(cell % I.n[o1]);
                c[o2] = (int)(cell / I.n[o1]);
                c[d] = mm == 0 ? -1 - j : I.n[d] + j;
                long long const idx = padIndex<DIM>(I, c[0], c[1], c[2]);
                T* const base = reinterpret_cast<T*>(I.buf[b]);
#pragma unroll
                for (int f = 0; f < 5; ++f) base[f * I.plane + idx] = (T)v[f];
            }
        }
    }
}

// The linear / quadratic boundaries (gridsolver.lua:783-858) of one
// instance's buffer: each ghost from the two (three) cells inside it, filled
// outward (j = 0 then 1, the min side before the max side as the reference's
// boundary kernel does), on the lines through the interior (corner ghosts are
// never read by the dimension-split stencil).  Lines are spread over `nthr`
// threads starting at `tid`.
template <typename T, int DIM>
__device__ void extrapGhosts(const DevInst& I, T* base, long long tid, long long nthr) {
#pragma unroll 1
    for (int d = 0; d < DIM; ++d) {
        int const lo = I.bc[2 * d], hi = I.bc[2 * d + 1];
        bool const xlo = lo == HC_BOUNDARY_LINEAR || lo == HC_BOUNDARY_QUADRATIC;
        bool const xhi = hi == HC_BOUNDARY_LINEAR || hi == HC_BOUNDARY_QUADRATIC;
        if (!xlo && !xhi) continue;
        int const o1 = (d + 1) % 3, o2 = (d + 2) % 3;
        int const n1 = o1 < DIM ? I.n[o1] : 1, n2 = o2 < DIM ? I.n[o2] : 1, N = I.n[d];
        for (long long line = tid; line < (long long)n1 * n2; line += nthr) {
            int c[3];
            c[o1] = (int)(line % n1);
            c[o2] = (int)(line / n1);
            auto at = [&](int x) -> long long {
                c[d] = x;
                return padIndex<DIM>(I, c[0], c[1], c[2]);
            };
            for (int j = 0; j < kG; ++j) {
                for (int mm = 0; mm < 2; ++mm) {
                    int const method = mm == 0 ? lo : hi;
                    if (method != HC_BOUNDARY_LINEAR && method != HC_BOUNDARY_QUADRATIC) continue;
                    int const s = mm == 0 ? -1 : 1;           // outward
                    int const g = mm == 0 ? -1 - j : N + j;    // the ghost
                    long long const id = at(g), i1 = at(g - s), i2 = at(g - 2 * s), i3 = at(g - 3 * s);
#pragma unroll
                    for (int f = 0; f < 5; ++f) {
                        T const a1 = base[f * I.plane + i1], a2 = base[f * I.plane + i2];
                        base[f * I.plane + id] = method == HC_BOUNDARY_LINEAR
                                                     ? T(2) * a1 - a2
                                                     : T(3) * a1 - T(3) * a2 + base[f * I.plane + i3];
                    }
                }
            }
        }
    }
}

// extrapGhosts of one instance (admission, resetState, boundary()).
template <typename T, int DIM>
__global__ void k_extrap_slot(const DevInst* inst, int slot, int buf) {
    const DevInst& I = inst[slot];
    extrapGhosts<T, DIM>(I, reinterpret_cast<T*>(I.buf[buf]), blockIdx.x * (long long)blockDim.x + threadIdx.x,
                         (long long)gridDim.x * blockDim.x);
}

// extrapGhosts of the output of a stage on every stepping instance of this
// dimension (grid.y = slots); state buffer `outBuf` of the plan, rotated per slot.
template <typename T, int DIM>
__global__ void k_extrap_stage(const DevInst* inst, const DevCtl* ctl, int nslots, int outBuf, int rotBuf) {
    for (int slot = blockIdx.y; slot < nslots; slot += gridDim.y) {
        const DevInst& I = inst[slot];
        if (I.dim != DIM || !ctl[slot].stepping) continue;
        int const b = slotBuf(outBuf, ctl[slot].rot, rotBuf);
        extrapGhosts<T, DIM>(I, reinterpret_cast<T*>(I.buf[b]), blockIdx.x * (long long)blockDim.x + threadIdx.x,
                             (long long)gridDim.x * blockDim.x);
    }
}

template <typename T, int DIM, bool EXACT>
__global__ void k_constrain(const DevInst* inst, int slot, int buf) {
    const DevInst& I = inst[slot];
    TileK<T> K;
    makeTileK<T>(K, I, nullptr, nullptr, 0, 0);
    T* base = reinterpret_cast<T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
        long long const idx = padIndex<DIM>(I, gx, gy, gz);
        T u[5];
        for (int f = 0; f < 5; ++f) u[f] = base[f * I.plane + idx];
        constrainCell<T, EXACT>(u, K);
        for (int f = 0; f < 5; ++f) base[f * I.plane + idx] = u[f];
    }
}

// calcDT of one slot's current state into ctl.dtmin[ctl.par] (reset first by the host).
template <typename T, int DIM, bool EXACT>
__global__ void k_calc_dt(const DevInst* inst, DevCtl* ctl, int slot, int buf) {
    const DevInst& I = inst[slot];
    TileK<T> K;
    makeTileK<T>(K, I, nullptr, nullptr, 0, 0);
    const T* base = reinterpret_cast<const T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    double m = __longlong_as_double((long long)kInfBits);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
        long long const idx = padIndex<DIM>(I, gx, gy, gz);
        T u[5];
        for (int f = 0; f < 5; ++f) u[f] = base[f * I.plane + idx];
        m = fmin(m, (double)dtCell<T, EXACT, DIM>(u, K, I));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m < __longlong_as_double((long long)kInfBits))
        atomicMin(&ctl[slot].dtmin[ctl[slot].par], (unsigned long long)__double_as_longlong(m));
}

// Interior <-> staging transfer with layout conversion (dir 0: staging -> grid)
// of interior cell k of n.
template <typename T, int DIM>
__device__ __forceinline__ void xferCell(const DevInst& I, T* base, void* staging, int layout, int dir, long long n,
                                         long long k) {
    int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
    long long const idx = padIndex<DIM>(I, gx, gy, gz);
    for (int f = 0; f < 5; ++f) {
        T* g = base + f * I.plane + idx;
        if (layout == HC_LAYOUT_AOS6_F64) {
            double* h = (double*)staging + 6 * k + f;
            if (dir == 0) *g = (T)*h; else *h = (double)*g;
        } else if (layout == HC_LAYOUT_SOA5_F64) {
            double* h = (double*)staging + f * n + k;
            if (dir == 0) *g = (T)*h; else *h = (double)*g;
        } else {
            float* h = (float*)staging + f * n + k;
            if (dir == 0) *g = (T)*h; else *h = (float)*g;
        }
    }
    if (layout == HC_LAYOUT_AOS6_F64 && dir == 1) ((double*)staging)[6 * k + 5] = 0.;
}

template <typename T, int DIM>
__global__ void k_xfer(const DevInst* inst, int slot, int buf, void* staging, int layout, int dir) {
    const DevInst& I = inst[slot];
    T* base = reinterpret_cast<T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        xferCell<T, DIM>(I, base, staging, layout, dir, n, k);
}

// The instances of one batched set-up or gather launch: job j is state
// buffer buf[j] of instance slot[j] with host-side buffer host[j] (page-locked
// memory mapped for the device, or staging), worked on by blocks first[j] ..
// first[j+1]-1, each taking kJobCells consecutive interior cells.  Passed by
// value (under 4 KB).
constexpr int kXferJobs = 120;
constexpr int kJobCells = 1024;
struct XferJobs {
    int n;
    int slot[kXferJobs];
    int buf[kXferJobs];
    int first[kXferJobs + 1];
    void* host[kXferJobs];
};

// The job of block b: the last j with first[j] <= b.
__device__ __forceinline__ int jobOf(const XferJobs& J, int b) {
    int lo = 0, hi = J.n - 1;
    while (lo < hi) {
        int const mid = (lo + hi + 1) >> 1;
        if (J.first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// k_xfer over the instances of J, one launch: block b moves kJobCells cells of
// its job (the same per-cell transfer).
template <typename T, int DIM>
__global__ void k_xfer_many(const DevInst* inst, const __grid_constant__ XferJobs J, int layout, int dir) {
    int const j = jobOf(J, blockIdx.x);
    const DevInst& I = inst[J.slot[j]];
    T* base = reinterpret_cast<T*>(I.buf[J.buf[j]]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    long long const k0 = (long long)(blockIdx.x - J.first[j]) * kJobCells;
    long long const k1 = k0 + kJobCells < n ? k0 + kJobCells : n;
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) xferCell<T, DIM>(I, base, J.host[j], layout, dir, n, k);
}

// The two layers next to face (axis, side) of one slot's buffer, as AoS-6
// doubles (ePot 0) x-fastest over the 2-layer slab, to staging (dir 1: the
// two interior layers next to the face) or from it (dir 0: the two ghost
// layers beyond the face).  A grid cut into slabs across ranks exchanges
// these between neighbours before every stage.
template <typename T, int DIM>
__global__ void k_slab(const DevInst* inst, int slot, int buf, int axis, int side, int dir, double* staging) {
    const DevInst& I = inst[slot];
    T* base = reinterpret_cast<T*>(I.buf[buf]);
    int ext[3] = {I.n[0], I.n[1], I.n[2]};
    ext[axis] = kG;
    long long const n = (long long)ext[0] * ext[1] * ext[2];
    int const N = I.n[axis];
    // first layer's coordinate along the axis
    int const c0 = dir ? (side ? N - kG : 0) : (side ? N : -kG);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        int c[3] = {(int)(k % ext[0]), (int)((k / ext[0]) % ext[1]), (int)(k / ((long long)ext[0] * ext[1]))};
        c[axis] += c0;
        long long const idx = padIndex<DIM>(I, c[0], c[1], c[2]);
        double* h = staging + 6 * k;
        if (dir) {
            for (int f = 0; f < 5; ++f) h[f] = (double)base[f * I.plane + idx];
            h[5] = 0.;
        } else {
            for (int f = 0; f < 5; ++f) base[f * I.plane + idx] = (T)h[f];
        }
    }
}

// A state set-up in one pass (admission, resetState, setState): staging ->
// interior with the layout conversion of k_xfer, constrainU when `reset`, the
// ghosts that copy one interior cell (periodic / mirror / freeflow) and the
// CFL min of the cell into ctl.dtmin[ctl.par] (reset to +inf beforehand).
// Every step reads and writes only its own cell's values, so the result is
// that of k_xfer, k_constrain, k_fill_ghosts and k_calc_dt run in turn; the
// linear / quadratic ghosts (k_extrap_slot) read neighbours and follow it.
// One cell of the set-up pass (interior cell k of n); returns its CFL dt.
template <typename T, int DIM, bool EXACT>
__device__ __forceinline__ double loadCell(const DevInst& I, const TileK<T>& K, T* base, const void* staging,
                                           int layout, int reset, long long n, long long k) {
    int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
    long long const idx = padIndex<DIM>(I, gx, gy, gz);
    T u[5];
    for (int f = 0; f < 5; ++f) {
        if (layout == HC_LAYOUT_AOS6_F64) u[f] = (T)((const double*)staging)[6 * k + f];
        else if (layout == HC_LAYOUT_SOA5_F64) u[f] = (T)((const double*)staging)[f * n + k];
        else u[f] = (T)((const float*)staging)[f * n + k];
    }
    if (reset) constrainCell<T, EXACT>(u, K);
    for (int f = 0; f < 5; ++f) base[f * I.plane + idx] = u[f];
    bool edge = false;
    int const g[3] = {gx, gy, gz};
    for (int d = 0; d < DIM; ++d) edge |= g[d] < 2 || g[d] >= I.n[d] - 2;
    if (edge) scatterGhosts<T, DIM>(I, base, gx, gy, gz, u);
    return (double)dtCell<T, EXACT, DIM>(u, K, I);
}

// The warps' CFL minima into the slot's dtmin[par].
__device__ __forceinline__ void dtminToSlot(DevCtl* ctl, int slot, double m) {
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m < __longlong_as_double((long long)kInfBits))
        atomicMin(&ctl[slot].dtmin[ctl[slot].par], (unsigned long long)__double_as_longlong(m));
}

template <typename T, int DIM, bool EXACT>
__global__ void k_load_state(const DevInst* inst, DevCtl* ctl, int slot, int buf, const void* staging, int layout,
                             int reset) {
    const DevInst& I = inst[slot];
    TileK<T> K;
    makeTileK<T>(K, I, nullptr, nullptr, 0, 0);
    T* base = reinterpret_cast<T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    double m = __longlong_as_double((long long)kInfBits);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        m = fmin(m, loadCell<T, DIM, EXACT>(I, K, base, staging, layout, reset, n, k));
    dtminToSlot(ctl, slot, m);
}

// k_load_state over the instances of J, one launch: block b sets up
// kJobCells cells of its job (the same per-cell pass).
template <typename T, int DIM, bool EXACT>
__global__ void k_load_many(const DevInst* inst, DevCtl* ctl, const __grid_constant__ XferJobs J, int layout,
                            int reset) {
    int const j = jobOf(J, blockIdx.x);
    int const slot = J.slot[j];
    const DevInst& I = inst[slot];
    TileK<T> K;
    makeTileK<T>(K, I, nullptr, nullptr, 0, 0);
    T* base = reinterpret_cast<T*>(I.buf[J.buf[j]]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    long long const k0 = (long long)(blockIdx.x - J.first[j]) * kJobCells;
    long long const k1 = k0 + kJobCells < n ? k0 + kJobCells : n;
    double m = __longlong_as_double((long long)kInfBits);
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x)
        m = fmin(m, loadCell<T, DIM, EXACT>(I, K, base, J.host[j], layout, reset, n, k));
    dtminToSlot(ctl, slot, m);
}

// Kahan-compensated FP64 sums of the 5 fields times the cell volume; one
// partial per block, combined on the host in block order.
template <typename T, int DIM>
__global__ void k_sums(const DevInst* inst, int slot, int buf, double vol, double* partial) {
    const DevInst& I = inst[slot];
    const T* base = reinterpret_cast<const T*>(I.buf[buf]);
    long long const n = (long long)I.n[0] * I.n[1] * I.n[2];
    double s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        int const gx = (int)(k % I.n[0]), gy = (int)((k / I.n[0]) % I.n[1]), gz = (int)(k / ((long long)I.n[0] * I.n[1]));
        long long const idx = padIndex<DIM>(I, gx, gy, gz);
        for (int f = 0; f < 5; ++f) {
            double const y = (double)base[f * I.plane + idx] * vol - c[f];
            double const tt = s[f] + y;
            c[f] = (tt - s[f]) - y;
            s[f] = tt;
        }
    }
    __shared__ double sh[5][256];
    for (int f = 0; f < 5; ++f) sh[f][threadIdx.x] = s[f];
    __syncthreads();
    if (threadIdx.x < 5) {
        int const f = threadIdx.x;
        double sm = 0, cc = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            double const y = sh[f][k] - cc;
            double const tt = sm + y;
            cc = (tt - sm) - y;
            sm = tt;
        }
        partial[5 * blockIdx.x + f] = sm;
    }
}

// ---------------------------------------------------------------------------
// launcher registry
// ---------------------------------------------------------------------------

struct StageLauncher {
    int precision;   // HC_F32_FUSED / HC_F64_FUSED
    int dim;
    int recon;       // HC_RECON_PLM_* compiled in, 0 (none), or -1 (any PLM kind, read at run time)
    bool lim;
    int slope;       // slope limiter compiled in, or -1 (any, dispatched at run time)
    int variant;     // tile-shape candidate index
    int tx, ty, tz, nthreads;
    int seg, unroll, min_ctas;   // segment length, sliding-window unroll (0: full), CTAs per SM compiled for
    int lanes;                   // lines per thread (2: packed FP32 pairs)
    int flux;                    // HC_FLUX_* compiled in, or -1 (any: read at run time)
    int box[3];                  // extents of the TMA box of the stage's input (x, y, z; the fields follow)
    int march;                   // 1: a marching kernel (one warp per strip item, work counter)
    size_t smem;
    void (*launch)(const StageArgs& a, int slopeLim, int fluxLim, int grid, cudaStream_t s);
    int (*occupancy)();   // CTAs per SM (sets the smem attribute first); <= 0 on error
};

struct AuxLauncher {
    int precision;
    int dim;
    void (*fill_ghosts)(const DevInst* inst, int slot, int buf, cudaStream_t s);
    void (*constrain)(const DevInst* inst, int slot, int buf, cudaStream_t s);
    void (*calc_dt)(const DevInst* inst, DevCtl* ctl, int slot, int buf, cudaStream_t s);
    // k_xfer over `cells` interior cells
    void (*xfer)(const DevInst* inst, int slot, int buf, void* staging, int layout, int dir, long long cells,
                 cudaStream_t s);
    // k_load_state over `cells` interior cells
    void (*load)(const DevInst* inst, DevCtl* ctl, int slot, int buf, const void* staging, int layout, int reset,
                 long long cells, cudaStream_t s);
    // k_load_many / k_xfer_many over the jobs of J (J.first[J.n] blocks)
    void (*load_many)(const DevInst* inst, DevCtl* ctl, const XferJobs& J, int layout, int reset, cudaStream_t s);
    void (*xfer_many)(const DevInst* inst, const XferJobs& J, int layout, int dir, cudaStream_t s);
    void (*extrap_slot)(const DevInst* inst, int slot, int buf, cudaStream_t s);
    void (*sums)(const DevInst* inst, int slot, int buf, double vol, double* partial, int blocks, cudaStream_t s);
    // linear / quadratic ghosts of a stage's output on every stepping instance of this dimension
    void (*extrap_stage)(const DevInst* inst, const DevCtl* ctl, int nslots, int out_buf, int rot_buf, cudaStream_t s);
    // k_fixed_ghosts on the first nbufs state buffers
    void (*fixed_ghosts)(const DevInst* inst, int slot, int nbufs, cudaStream_t s);
    // k_slab over `cells` slab cells
    void (*slab)(const DevInst* inst, int slot, int buf, int axis, int side, int dir, double* staging, long long cells,
                 cudaStream_t s);
};

void register_launchers(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux);

}  // namespace fz
}  // namespace hc
