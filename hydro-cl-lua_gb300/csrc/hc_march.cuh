// hc_march.cuh -- the 2D marching stage kernel (FP32 fast form, "plm cons").
//
// One warp advances one strip of a grid: 30 interior columns (lanes 1..30;
// lanes 0 and 31 carry the cells beside the strip) over a segment of seg
// rows (H, the schedule's segment, unless the host shortens the segments of a
// launch whose items would leave warps idle).
// The warp marches up the segment one row per step.  The cells come from the
// chunk buffers in shared memory (rows r-1 .. r+1 at every step); a lane
// carries in registers the cell below's y-side R state and y-face flux and the
// row below's x-flux difference.  Each step of a lane:
//   * the x and y half slopes of its cell, evaluated together on FP32
//     register pairs (.x: the x axis, .y: the y axis; pair j holds global
//     field j on x and the y interface frame's field j on y, the order the
//     Roe lanes take);
//   * the Roe flux of its cell's left x face (the left neighbour's R state
//     comes by warp shuffle) and of its cell's lower y face, together on
//     register pairs;
//   * the x flux difference of its cell (the right face flux by shuffle) and
//     the y flux difference of the cell below, which is then finished:
//     Runge-Kutta combination, constrainU, store, ghost copies and, on the
//     last stage, its CFL dt.
// So every slope and every face flux is computed once per strip, except the
// two columns beside the strip and the two rows beside the segment.  No
// shared-memory accumulator and no block-wide barrier exist: the warp's rows
// arrive in chunks of C rows by TMA (cp.async.bulk.tensor, one mbarrier per
// chunk buffer, NB buffers in flight), and the warp takes its next item from
// a work counter when it finishes one.
//
// The arithmetic is that of the tile kernel operation for operation
// (hc_lanes.cuh: the same slope, flux, combination, constrainU and dt
// functions; the packed forms round each lane exactly as the scalar ones), so
// both kernels produce identical bits.
#pragma once

#include "hc_fused.cuh"

namespace hc {
namespace fz {

constexpr int kStripW = 30;     // interior columns of a strip (one warp)
constexpr int kMarchBW = 40;    // box width: 34 columns + the 16-byte alignment slack of the TMA x coordinate

template <int NW, int C, int NB>
struct MarchCfg {
    static_assert(C % 4 == 0, "chunk buffers must be 128-byte multiples (5 x C x 160 B)");
    static_assert(NB >= 2, "at least two chunk buffers");
    static constexpr int BUFF = 5 * C * kMarchBW;               // floats per chunk buffer [field][row][column]
    static constexpr int WARPF = NB * BUFF;                     // floats per warp
    static constexpr size_t kBarOff = (size_t)NW * WARPF * 4;   // then NB mbarriers per warp
    static constexpr size_t SMEM = kBarOff + (size_t)NW * NB * 8;
    static constexpr unsigned BYTES = (unsigned)(BUFF * 4);
};

// The epilogue forms the launcher compiles (EPI): 0 reads the stage's
// structure at run time; the others have it fixed -- no stored derivatives
// and no beta terms, a current-derivative term, and the alpha terms
//   1: the staged input alone (forward Euler, the first stage of RK2 / RK3-TVD)
//   2: one state from global memory, on the step's last stage (the midpoint
//      RK2's second stage): the CFL dt without a run-time test
//   3: one state from global memory, then the staged input (the later stages
//      of RK2-TVD and RK3-TVD)
inline int marchEpi(const StageDev& s) {
    if (s.n_beta != 0 || s.store_deriv >= 0 || s.beta_cur == 0.) return 0;
    if (s.n_alpha == 1) return s.alpha_buf[0] == s.in_buf ? 1 : (s.last ? 2 : 0);
    if (s.n_alpha == 2 && s.alpha_buf[0] != s.in_buf && s.alpha_buf[1] == s.in_buf) return 3;
    return 0;
}

// The y axis' interface frame takes (rho, m.y, m.z, m.x, E): global field g of
// the y lane sits at frame index kYFrame[g].
__device__ __forceinline__ constexpr int yFrameOf(int g) { return g == 0 ? 0 : (g == 4 ? 4 : (g == 1 ? 3 : g - 1)); }
// and frame index j holds global field yGlobalOf(j)
__device__ __forceinline__ constexpr int yGlobalOf(int j) { return j == 0 ? 0 : (j == 4 ? 4 : (j == 3 ? 1 : j + 1)); }

// The ghost copies a finished 2D cell (x, y) at padded index idx makes
// (gridsolver.lua:638-780): periodic wraps, mirror reflects with the normal
// momentum negated, freeflow repeats the edge cell -- the copies of
// scatterGhosts, addressed by their offset from idx (a row is px elements).
__device__ __forceinline__ void marchGhosts(float* out, long long plane, int px, int nx, int ny, const int* bc, int x,
                                            int y, long long idx, const float* u) {
    auto put = [&](long long off, int negf) {
#pragma unroll
        for (int f = 0; f < 5; ++f) out[f * plane + idx + off] = f == negf ? -1.f * u[f] : u[f];
    };
    if (x < 2 || x >= nx - 2) {
        int const lo = bc[0], hi = bc[1];
        if (lo == HC_BOUNDARY_PERIODIC && x >= nx - 2) put(-nx, -1);
        if (lo == HC_BOUNDARY_MIRROR && x <= 1) put(-1 - 2 * x, 1);
        if (lo == HC_BOUNDARY_FREEFLOW && x == 0) { put(-1, -1); put(-2, -1); }
        if (hi == HC_BOUNDARY_PERIODIC && x <= 1) put(nx, -1);
        if (hi == HC_BOUNDARY_MIRROR && x >= nx - 2) put(2 * nx - 1 - 2 * x, 1);
        if (hi == HC_BOUNDARY_FREEFLOW && x == nx - 1) { put(1, -1); put(2, -1); }
    }
    if (y < 2 || y >= ny - 2) {
        int const lo = bc[2], hi = bc[3];
        long long const r = px;
        if (lo == HC_BOUNDARY_PERIODIC && y >= ny - 2) put(-ny * r, -1);
        if (lo == HC_BOUNDARY_MIRROR && y <= 1) put((-1 - 2 * y) * r, 2);
        if (lo == HC_BOUNDARY_FREEFLOW && y == 0) { put(-r, -1); put(-2 * r, -1); }
        if (hi == HC_BOUNDARY_PERIODIC && y <= 1) put(ny * r, -1);
        if (hi == HC_BOUNDARY_MIRROR && y >= ny - 2) put((2 * ny - 1 - 2 * y) * r, 2);
        if (hi == HC_BOUNDARY_FREEFLOW && y == ny - 1) { put(r, -1); put(2 * r, -1); }
    }
}

template <int NW, int H, int C, int NB, int SLOPE, int OCC, int EPI>
__global__ void __launch_bounds__(NW * 32, OCC) k_march2(const __grid_constant__ StageArgs a, int slopeLim, int fluxLim) {
    using Cfg = MarchCfg<NW, C, NB>;
    (void)fluxLim;
    extern __shared__ __align__(128) unsigned char smem[];
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* const wb = reinterpret_cast<float*>(smem) + (size_t)warp * Cfg::WARPF;
    uint64_t* const bars = reinterpret_cast<uint64_t*>(smem + Cfg::kBarOff) + warp * NB;
    if (lane == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) mbar_init(&bars[b], 1);
        fence_barrier_init();
    }
    __syncwarp();
    unsigned phase = 0;   // bit b: parity of the next completion of buffer b
    int const nitems = *a.nitems;
    const StageDev& st = a.st;
    constexpr unsigned FULL = 0xffffffffu;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.work, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        int4 const it = a.items[item];
        const DevInst& I = a.inst[it.x];
        DevCtl* const ctl = a.ctl + it.x;
        if (!ctl->stepping) continue;
        int const rot = ctl->rot;
        int const inBuf = slotBuf(st.in_buf, rot, a.rot_buf);
        Geo const geo = geoOf(I);
        int const nx = geo.n[0], ny = geo.n[1];
        int const seg = *a.seg;   // read per item: nothing holds it across the march
        int const x0 = it.y * kStripW, y0 = it.z * seg;
        int const rows = ny - y0 < seg ? ny - y0 : seg;
        int const nrows = rows + 4;                  // box rows y0-2 .. y0+rows+1
        int const nchunks = (nrows + C - 1) / C;
        // padded column of the strip's first box column (cell x0-2), rounded
        // down to 4 elements (16 bytes) for the TMA x coordinate
        int const pa = x0 & ~3;
        const CUtensorMap* const map = a.tmaps + (size_t)it.x * kMaxBufs + inBuf;

        // chunk k (rows y0-2+kC ...) into buffer k % NB
        auto issue = [&](int k) {
            int const b = k % NB;
            fence_proxy_async();
            mbar_arrive_expect_tx(&bars[b], Cfg::BYTES);
            tma_load<3>(wb + b * Cfg::BUFF, map, pa, y0 + k * C, 0, 0, &bars[b]);
        };
        __syncwarp();   // every lane is done with the buffers of the previous item
        if (lane == 0)
            for (int k = 0; k < NB && k < nchunks; ++k) issue(k);
        __syncwarp();
        int ready = 0;   // chunks waited for
        bool timedOut = false;
        auto waitChunk = [&]() {
            int const b = ready % NB;
            bool ok = a.force_timeout ? false : mbar_wait_bounded(&bars[b], (phase >> b) & 1u, kSpinLimit);
            ok = __shfl_sync(FULL, ok, 0);   // lane 0 decides for the warp
            if (!ok) {
                // record it; give the copy a second bounded chance to land
                // before the warp leaves its buffers
                if (lane == 0) { atomicOr(a.err, DEV_TIMEOUT); atomicOr(&ctl->status, DEV_TIMEOUT); }
                mbar_wait_bounded(&bars[b], (phase >> b) & 1u, kSpinLimit);
                timedOut = true;
            }
            phase ^= 1u << b;
            ++ready;
        };
        // box element of field f, box row i (0: y0-2), box column c
        auto at = [&](int f, int i, int c) -> float {
            return wb[((i / C) % NB) * Cfg::BUFF + (f * C + i % C) * kMarchBW + c];
        };

        TileK<float> K;
        makeTileK<float>(K, I, ctl, &st, slopeLim, 0, HC_FLUX_ROE, 2, HC_RECON_PLM_CONS);
        lanes::Eos const le{K.fe.gamma, K.fe.g1, K.fe.rhoMin, K.fe.PMin, K.fe.hllcMethod, K.invg1, K.re.recon,
                             (float)K.fe.entropyFactor};
        int const slim = SLOPE >= 0 ? SLOPE : K.fe.slopeLimiter;
        float2 const area = make_float2(K.area[0], K.area[1]);
        bool const skipX = K.skip[0], skipY = K.skip[1], zeroX = K.zero[0], zeroY = K.zero[1];
        float const cbcur = K.cbcur;
        bool const useCur = K.useCur;

        // the lane's column; lanes beyond the grid's last ghost column repeat
        // it (finite states, never stored)
        int const x = x0 - 1 + lane;
        bool const inCols = lane >= 1 && lane <= kStripW && x < nx;
        int const xc = x < nx ? x : nx;
        int const col = xc + 2 - pa;   // box column of the lane's cell

        float* const out = reinterpret_cast<float*>(I.buf[slotBuf(st.out_buf, rot, a.rot_buf)]);
        float* const dstore = st.store_deriv >= 0 ? reinterpret_cast<float*>(I.dbuf[st.store_deriv]) : nullptr;
        // the first Runge-Kutta state the epilogue reads from global memory
        // (not the staged input): read one step ahead into registers, so its
        // latency overlaps a step's flux arithmetic
        int a0 = -1;
        const float* a0src = nullptr;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            if (m >= st.n_alpha) break;
            int const b = slotBuf(st.alpha_buf[m], rot, a.rot_buf);
            if (b != inBuf && a0 < 0) {
                a0 = m;
                a0src = reinterpret_cast<const float*>(I.buf[b]);
            }
        }
        // padded index of cell (x, y0); row r adds r * px
        long long const idx0 = padIndex<2>(geo, xc, y0, 0);
        float pre[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) pre[f] = 0.f;
        if (a0 >= 0) {
#pragma unroll
            for (int f = 0; f < 5; ++f) pre[f] = a0src[f * geo.plane + idx0];
        }

        float dtmin = fast::M<float>::inf();
        bool bad = false;

        // carried by the march (the cells themselves are re-read from shared
        // memory, which holds rows r-1 .. r+1 at every step)
        float Ry[5];       // the y-side R state of cell (x, r-1), y interface frame
        float Fyp[5];      // the y flux at the lower face of cell (x, r-1), global frame
        float Dxp[5];      // the x flux difference of cell (x, r-1)
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            Ry[f] = 0.f;
            Fyp[f] = 0.f;
            Dxp[f] = 0.f;
        }
        waitChunk();   // box rows 0 and 1 (chunk 0)

        // step ir: r = y0 - 2 + ir, slopes of (x, r), the x face flux of row r,
        // the y face flux below (x, r), cell (x, r-1) finished from ir = 3 on
        // (every lane evaluates it; only the strip's own cells are stored)
        bool const edgeX = x0 < 2 || x0 + kStripW > nx - 2;   // the strip holds cells with x ghost copies
        float const arx = K.area[0], ary = K.area[1];
#pragma unroll 1
        for (int ir = 1; ir <= rows + 2; ++ir) {
            // step ir reads box rows ir - 1 .. ir + 1: chunk (ir - 1) / C - 1 is
            // no longer read, refill its buffer
            if ((ir - 1) % C == 0 && ir - 1 >= C) {
                int const k = (ir - 1) / C - 1 + NB;
                __syncwarp();
                if (lane == 0 && k < nchunks) issue(k);
            }
            if (ready <= (ir + 1) / C) {
                do waitChunk();
                while (ready <= (ir + 1) / C);
                if (timedOut) break;
            }
            // the lane's column in box rows ir - 1, ir, ir + 1
            const float* const rm = wb + ((ir - 1) / C % NB) * Cfg::BUFF + ((ir - 1) % C) * kMarchBW + col;
            const float* const r0 = wb + (ir / C % NB) * Cfg::BUFF + (ir % C) * kMarchBW + col;
            const float* const rp = wb + ((ir + 1) / C % NB) * Cfg::BUFF + ((ir + 1) % C) * kMarchBW + col;
            // x and y half slopes of (x, r), L = U - h, R = U + h, paired in
            // the interface frames: pair j holds global field j on the x axis
            // and field yGlobalOf(j) on the y axis, as the Roe lanes take them
            float2 L[5], R[5];
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                int const g = yGlobalOf(j);
                float2 const c = make_float2(r0[j * C * kMarchBW], r0[g * C * kMarchBW]);
                float2 const dL = lanes::sub(c, make_float2(r0[j * C * kMarchBW - 1], rm[g * C * kMarchBW]));
                float2 const dR = lanes::sub(make_float2(r0[j * C * kMarchBW + 1], rp[g * C * kMarchBW]), c);
                float2 const h = lanes::halfSlope<SLOPE>(dL, dR, slim);
                L[j] = lanes::sub(c, h);
                R[j] = lanes::add(c, h);
            }
            if (ir >= 2) {
                // faces: x (left neighbour's R | own L), y (own R one row down | own L)
                lanes::C5<float2> UL, UR;
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    UL.u[j] = make_float2(__shfl_up_sync(FULL, R[j].x, 1), Ry[j]);
                    UR.u[j] = L[j];
                }
                float2 F[5];
                bool const plain = lanes::roeUp2(F, le, UL, UR);
                if (!__all_sync(FULL, plain)) {
                    // a lane somewhere in the warp has a vacuum side or a
                    // degenerate average: every lane evaluates both faces in
                    // the scalar form (the same bits where the packed form held)
#pragma unroll 1
                    for (int k = 0; k < 2; ++k) {
                        lanes::C5<float> l, r;
#pragma unroll
                        for (int j = 0; j < 5; ++j) {
                            l.u[j] = lanes::lane(UL.u[j], k);
                            r.u[j] = lanes::lane(UR.u[j], k);
                        }
                        float fk[5];
                        lanes::roe<float>(fk, le, l, r);
#pragma unroll
                        for (int j = 0; j < 5; ++j) lanes::setLane(F[j], k, fk[j]);
                    }
                }
                // calcDerivFromFlux: x difference of (x, r) (its right face flux
                // by shuffle), then the y difference of (x, r-1) added to its x
                // difference, each fma(FL - FR, area, deriv) rounded as written
                // (a face of no area has no flux)
                float deriv[5];
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    float const fx = zeroX ? 0.f : F[f].x;
                    float const fy = zeroY ? 0.f : F[yFrameOf(f)].y;
                    float const fxr = __shfl_down_sync(FULL, fx, 1);
                    deriv[f] = skipY ? Dxp[f] : __fmaf_rn(__fsub_rn(Fyp[f], fy), ary, Dxp[f]);
                    Dxp[f] = skipX ? 0.f : __fmaf_rn(__fsub_rn(fx, fxr), arx, 0.f);
                    Fyp[f] = fy;
                }
                if (ir >= 3) {
                    // cell (x, r-1): u = sum alpha_k u^(k) + sum (beta_k dt) L(u^(k)) + (beta_cur dt) deriv
                    int const yc = y0 - 3 + ir;
                    long long const idx = idx0 + (long long)(ir - 3) * geo.px;
                    float u[5];
                    if constexpr (EPI == 0) {
                    auto ldAlpha = [&](int m, float* v) {
                        int const b = slotBuf(st.alpha_buf[m], rot, a.rot_buf);
                        if (m == a0) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) v[f] = pre[f];
                        } else if (b == inBuf) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) v[f] = rm[f * C * kMarchBW];
                        } else {
                            const float* const src = reinterpret_cast<const float*>(I.buf[b]);
#pragma unroll
                            for (int f = 0; f < 5; ++f) v[f] = src[f * geo.plane + idx];
                        }
                    };
                    int const last = st.n_alpha - 1;
                    float p[5];
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        if (m == last) ldAlpha(m, p);
#pragma unroll
                    for (int f = 0; f < 5; ++f) u[f] = p[f];
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        if (m >= last) break;
                        float w[5];
                        ldAlpha(m, w);
#pragma unroll
                        for (int f = 0; f < 5; ++f) u[f] = lanes::fma(lanes::sub(w[f], p[f]), K.calpha[m], u[f]);
                    }
                    // the next step's cell
                    if (a0 >= 0) {
                        // (the segment's last row read again at its end: no branch)
                        const float* const pn = a0src + idx + (yc + 1 < y0 + rows ? geo.px : 0);
#pragma unroll
                        for (int f = 0; f < 5; ++f) pre[f] = pn[f * geo.plane];
                    }
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
                        if (m >= st.n_beta) break;
                        const float* const src = reinterpret_cast<const float*>(I.dbuf[st.beta_buf[m]]);
#pragma unroll
                        for (int f = 0; f < 5; ++f) u[f] = lanes::fma(src[f * geo.plane + idx], K.cbeta[m], u[f]);
                    }
                    if (useCur) {
#pragma unroll
                        for (int f = 0; f < 5; ++f) u[f] = lanes::fma(deriv[f], cbcur, u[f]);
                    }
                    } else {
                        // the stage's structure is fixed at compile time (the
                        // launcher picks the kernel): the same operations as
                        // above in the same order, without the run-time choices
                        if constexpr (EPI == 1) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) u[f] = rm[f * C * kMarchBW];
                        } else if constexpr (EPI == 2) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) u[f] = pre[f];
                        } else {
#pragma unroll
                            for (int f = 0; f < 5; ++f) {
                                float const pb = rm[f * C * kMarchBW];
                                u[f] = lanes::fma(lanes::sub(pre[f], pb), K.calpha[0], pb);
                            }
                        }
                        if constexpr (EPI != 1) {
                            // the next row's cell (the segment's last row read
                            // again at its end: no branch); issued a row ahead
                            // of its use, it needs no L2 prefetch besides
                            const float* const pn = a0src + idx + (yc + 1 < y0 + rows ? geo.px : 0);
#pragma unroll
                            for (int f = 0; f < 5; ++f) pre[f] = pn[f * geo.plane];
                        }
#pragma unroll
                        for (int f = 0; f < 5; ++f) u[f] = lanes::fma(deriv[f], cbcur, u[f]);
                    }
                    lanes::constrain<float>(u, le, K.invg1);
                    if (inCols) {
#pragma unroll
                        for (int f = 0; f < 5; ++f) out[f * geo.plane + idx] = u[f];
                        if (EPI == 0 && dstore) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) dstore[f * geo.plane + idx] = deriv[f];
                        }
                    }
                    // after constrainU a non-finite momentum shows in ETotal
                    bad |= inCols && !fast::M<float>::finite_(u[0] + u[4]);
                    // the same for every lane: a warp-uniform branch
                    if (__any_sync(FULL, edgeX || yc < 2 || yc >= ny - 2))
                        if (inCols) marchGhosts(out, geo.plane, geo.px, nx, ny, geo.bc, x, yc, idx, u);
                    if (EPI == 2 || st.last) {
                        float const dtc = lanes::dtCell<float, 2>(u, le, K.gdx);
                        if (inCols) dtmin = fast::tmin(dtmin, dtc);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < 5; ++j) Ry[j] = R[j].y;
        }
        if (timedOut) return;
        // one FP64 atomicMin per item for the next step's CFL dt
        if (EPI == 2 || st.last) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dtmin = fast::tmin(dtmin, __shfl_xor_sync(FULL, dtmin, o));
            double const m = (double)dtmin;
            if (lane == 0 && m < __longlong_as_double((long long)kInfBits))
                atomicMin(&ctl->dtmin[ctl->par ^ 1], (unsigned long long)__double_as_longlong(m));
        }
        if (__any_sync(FULL, bad) && lane == 0) atomicOr(&ctl->status, DEV_NONFINITE);
    }
}

}  // namespace fz
}  // namespace hc
