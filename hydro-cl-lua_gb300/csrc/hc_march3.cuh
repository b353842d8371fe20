// hc_march3.cuh -- the 3D marching stage kernel (FP32 fast form, "plm cons").
//
// One CTA advances one x-y tile of a 3D grid up a segment of seg planes
// along z (D, the schedule's segment, unless the host shortens the segments
// of a launch whose items would leave CTAs idle).  The tile is 30 columns wide (lanes 1..30 of every warp; lanes 0 and 31
// carry the columns beside it) and NWY - 1 rows high: warp w holds row
// y0 - 1 + w, so warp 0 carries the row below the tile.  The planes arrive
// one at a time by TMA (cp.async.bulk.tensor, box 40 x (NWY+3) x 1 x 5
// floats, one mbarrier per buffer, NB buffers in flight) into a ring the
// whole CTA reads.  Each step of the march, for plane p:
//   * every row takes the y half slopes of its cell and of the cell above it,
//     and the Roe flux of its cell's upper y face, which it publishes in
//     shared memory;
//   * the tile's rows also take the x and z half slopes of their cell and the
//     Roe fluxes of its left x face (the left lane's R state by warp shuffle)
//     and of the z face below it (the cell below's R state carried in
//     registers), the two together on FP32 register pairs;
//   * after one block barrier each tile row reads its lower y face flux (the
//     row below's upper one), keeps the x and y flux differences of plane p
//     in registers and finishes the cell of plane p - 1 with its z flux
//     difference: Runge-Kutta combination, constrainU, store, ghost copies
//     and, on the last stage, its CFL dt.
// So every face flux is computed once per tile (one y slope a cell is taken
// twice instead of exchanged, which would cost a second barrier), except the
// columns beside the tile and the planes beside the segment, and a plane's
// cells are read from HBM once (the box halo comes from L2: neighbouring
// tiles march the same planes at the same time).
//
// The arithmetic is that of the tile kernel operation for operation: the x,
// y and z flux differences accumulate in that order, each
// fma(FL - FR, area, acc) rounded as written, with the same slope, flux,
// combination, constrainU and dt functions, so both kernels produce
// identical bits.
#pragma once

#include "hc_march.cuh"

namespace hc {
namespace fz {

template <int NWY, int NB>
struct March3Cfg {
    static_assert(NWY >= 2 && NWY <= 32, "at least one tile row above the row below the tile");
    static_assert(NB >= 4, "planes p-1, p, p+1 in use and one in flight");
    static constexpr int ROWS = NWY + 3;                     // box rows y0-2 .. y0+NWY
    static constexpr int FS = ROWS * kMarchBW;               // floats of one field of a plane
    static constexpr int PLANEF = 5 * FS;                    // floats of one plane [field][row][column]
    static constexpr int BUFF = (PLANEF + 31) / 32 * 32;     // buffer stride, a multiple of 128 bytes
    static constexpr int XCH = NWY * 5 * 32;                 // floats of one face-flux array [warp][field][lane]
    static constexpr size_t kXchOff = (size_t)NB * BUFF * 4;
    static constexpr size_t kBarOff = kXchOff + (size_t)2 * XCH * 4;   // two, by step parity
    static constexpr size_t kItemOff = kBarOff + (size_t)NB * 8;
    static constexpr size_t SMEM = kItemOff + 16;
    static constexpr unsigned BYTES = (unsigned)(PLANEF * 4);
};

// The z axis' interface frame takes (rho, m.z, m.x, m.y, E): global field g of
// the z lane sits at frame index zFrameOf(g).
__device__ __forceinline__ constexpr int zFrameOf(int g) { return g == 0 ? 0 : (g == 4 ? 4 : (g == 3 ? 1 : g + 1)); }
// and frame index j holds global field zGlobalOf(j)
__device__ __forceinline__ constexpr int zGlobalOf(int j) { return j == 0 ? 0 : (j == 4 ? 4 : (j == 1 ? 3 : j - 1)); }

// The z ghost copies of a finished 3D cell at plane z, padded index idx (a
// plane is s elements): those of scatterGhosts along z.
__device__ __forceinline__ void marchGhostsZ(float* out, long long plane, long long s, int nz, const int* bc, int z,
                                             long long idx, const float* u) {
    auto put = [&](long long off, int negf) {
#pragma unroll
        for (int f = 0; f < 5; ++f) out[f * plane + idx + off] = f == negf ? -1.f * u[f] : u[f];
    };
    int const lo = bc[4], hi = bc[5];
    if (lo == HC_BOUNDARY_PERIODIC && z >= nz - 2) put(-nz * s, -1);
    if (lo == HC_BOUNDARY_MIRROR && z <= 1) put((-1 - 2 * z) * s, 3);
    if (lo == HC_BOUNDARY_FREEFLOW && z == 0) { put(-s, -1); put(-2 * s, -1); }
    if (hi == HC_BOUNDARY_PERIODIC && z <= 1) put(nz * s, -1);
    if (hi == HC_BOUNDARY_MIRROR && z >= nz - 2) put((2 * nz - 1 - 2 * z) * s, 3);
    if (hi == HC_BOUNDARY_FREEFLOW && z == nz - 1) { put(s, -1); put(2 * s, -1); }
}

template <int NWY, int D, int NB, int SLOPE, int OCC, int EPI>
__global__ void __launch_bounds__(NWY * 32, OCC) k_march3(const __grid_constant__ StageArgs a, int slopeLim, int fluxLim) {
    using Cfg = March3Cfg<NWY, NB>;
    constexpr int TR = NWY - 1;        // tile rows
    constexpr int FS = Cfg::FS;
    (void)fluxLim;
    extern __shared__ __align__(128) unsigned char smem[];
    float* const ring = reinterpret_cast<float*>(smem);
    // upper y face fluxes [parity][warp][field][lane]: written before a
    // step's barrier and read after it, a step's parity apart from the next
    // step's writes
    float* const FY = reinterpret_cast<float*>(smem + Cfg::kXchOff);
    uint64_t* const bars = reinterpret_cast<uint64_t*>(smem + Cfg::kBarOff);
    int* const itemSlot = reinterpret_cast<int*>(smem + Cfg::kItemOff);
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) mbar_init(&bars[b], 1);
        fence_barrier_init();
    }
    __syncthreads();
    unsigned phase = 0;   // bit b: parity of the next completion of buffer b
    int const nitems = *a.nitems;
    const StageDev& st = a.st;
    constexpr unsigned FULL = 0xffffffffu;

    for (;;) {
        // every thread is done with the previous item's buffers and slot
        __syncthreads();
        if (threadIdx.x == 0) *itemSlot = atomicAdd(a.work, 1);
        __syncthreads();
        int const item = *itemSlot;
        if (item >= nitems) break;
        int4 const it = a.items[item];
        const DevInst& I = a.inst[it.x];
        DevCtl* const ctl = a.ctl + it.x;
        if (!ctl->stepping) continue;
        int const rot = ctl->rot;
        int const inBuf = slotBuf(st.in_buf, rot, a.rot_buf);
        Geo const geo = geoOf(I);
        int const nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
        int const seg = *a.seg;   // read per item: nothing holds it across the march
        int const x0 = it.y * kStripW, y0 = it.z * TR, z0 = it.w * seg;
        int const planes = nz - z0 < seg ? nz - z0 : seg;
        int const nplanes = planes + 4;              // box planes z0-2 .. z0+planes+1
        int const pa = x0 & ~3;                      // padded column of cell x0-2, rounded down to 16 bytes
        const CUtensorMap* const map = a.tmaps + (size_t)it.x * kMaxBufs + inBuf;
        // box plane k (cell plane z0-2+k) into buffer k % NB; box row 0 is cell row y0-2
        auto issue = [&](int k) {
            int const b = k % NB;
            fence_proxy_async();
            mbar_arrive_expect_tx(&bars[b], Cfg::BYTES);
            tma_load<4>(ring + b * Cfg::BUFF, map, pa, y0, z0 + k, 0, &bars[b]);
        };
        if (threadIdx.x == 0)
            for (int k = 0; k < NB && k < nplanes; ++k) issue(k);
        int issued = nplanes < NB ? nplanes : NB;   // tracked alike by every thread
        int ready = 0;                               // planes waited for
        auto waitPlane = [&]() -> bool {
            int const b = ready % NB;
            bool ok = a.force_timeout ? false : mbar_wait_bounded(&bars[b], (phase >> b) & 1u, kSpinLimit);
            if (!ok) {
                // record it; give the copy a second bounded chance to land
                // before the CTA leaves its buffers
                atomicOr(a.err, DEV_TIMEOUT);
                atomicOr(&ctl->status, DEV_TIMEOUT);
                mbar_wait_bounded(&bars[b], (phase >> b) & 1u, kSpinLimit);
            }
            phase ^= 1u << b;
            ++ready;
            return ok;
        };

        TileK<float> K;
        makeTileK<float>(K, I, ctl, &st, slopeLim, 0, HC_FLUX_ROE, 2, HC_RECON_PLM_CONS);
        lanes::Eos const le{K.fe.gamma, K.fe.g1, K.fe.rhoMin, K.fe.PMin, K.fe.hllcMethod, K.invg1, K.re.recon,
                             (float)K.fe.entropyFactor};
        int const slim = SLOPE >= 0 ? SLOPE : K.fe.slopeLimiter;
        bool const skipX = K.skip[0], skipY = K.skip[1], skipZ = K.skip[2];
        bool const zeroX = K.zero[0], zeroY = K.zero[1], zeroZ = K.zero[2];
        float const arx = K.area[0], ary = K.area[1], arz = K.area[2];
        float const cbcur = K.cbcur;
        bool const useCur = K.useCur;

        // the thread's cell: column x (lanes beyond the grid's last ghost
        // column repeat it: finite states, never stored), row yw
        int const x = x0 - 1 + lane;
        bool const inCols = lane >= 1 && lane <= kStripW && x < nx;
        int const xc = x < nx ? x : nx;
        int const yw = y0 - 1 + warp;
        bool const faceRow = yw < ny;                 // takes the y face above its row
        bool const tileRow = warp >= 1 && yw < ny;    // finishes cells
        int const cell = (warp + 1) * kMarchBW + xc + 2 - pa;       // box offset of the cell within a field
        long long const ps = (long long)geo.px * geo.py;            // padded elements of a plane

        float* const out = reinterpret_cast<float*>(I.buf[slotBuf(st.out_buf, rot, a.rot_buf)]);
        float* const dstore = st.store_deriv >= 0 ? reinterpret_cast<float*>(I.dbuf[st.store_deriv]) : nullptr;
        // the first Runge-Kutta state the epilogue reads from global memory
        // (not the staged input): read one plane ahead into registers
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
        // padded index of cell (x, yw, z0); plane k adds k * ps
        long long const idx0 = padIndex<3>(geo, xc, tileRow ? yw : 0, z0);
        float pre[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) pre[f] = 0.f;
        if (a0 >= 0 && tileRow) {
#pragma unroll
            for (int f = 0; f < 5; ++f) pre[f] = a0src[f * geo.plane + idx0];
        }

        float dtmin = fast::M<float>::inf();
        bool bad = false;
        bool timedOut = false;
        bool const edgeXY = x0 < 2 || x0 + kStripW > nx - 2 || yw < 2 || yw >= ny - 2;

        // carried by the march
        float Rz[5];       // the z-side R state of the cell below (plane p-1), z interface frame
        float Fzp[5];      // the z flux at the lower face of the cell below
        float Dxy[5];      // the x and y flux differences of the cell below
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            Rz[f] = 0.f;
            Fzp[f] = 0.f;
            Dxy[f] = 0.f;
        }

        // step iz: plane p = z0 - 2 + iz; the cell of plane p - 1 is finished
        // from iz = 3 on
#pragma unroll 1
        for (int iz = 1; iz <= planes + 2; ++iz) {
            bool ok = true;
            while (ready <= iz + 1) ok &= waitPlane();
            const float* const pm = ring + ((iz - 1) % NB) * Cfg::BUFF + cell;
            const float* const p0 = ring + (iz % NB) * Cfg::BUFF + cell;
            const float* const pp = ring + ((iz + 1) % NB) * Cfg::BUFF + cell;
            // y half slopes, L = U - h, R = U + h: the row's cell (its R) and
            // the cell above (its L)
            float Ry[5], Lya[5];
            if (faceRow) {
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    float const u0 = p0[f * FS];
                    float const ua = p0[f * FS + kMarchBW];
                    float const hy = lanes::halfSlope<SLOPE>(lanes::sub(u0, p0[f * FS - kMarchBW]),
                                                             lanes::sub(ua, u0), slim);
                    float const hya = lanes::halfSlope<SLOPE>(lanes::sub(ua, u0),
                                                              lanes::sub(p0[f * FS + 2 * kMarchBW], ua), slim);
                    Ry[f] = lanes::add(u0, hy);
                    Lya[f] = lanes::sub(ua, hya);
                }
            }
            float* const fyp = FY + (iz & 1) * Cfg::XCH;
            float fy[5];
            if (iz >= 2 && faceRow) {
                // the upper y face: own R | the cell above's L; the lean form,
                // the general one on a lane without the plain Roe average
                lanes::C5<float> ul, ur;
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    int const j = yFrameOf(f);
                    ul.u[j] = Ry[f];
                    ur.u[j] = Lya[f];
                }
                float F[5];
                if (!lanes::roeUp<float>(F, le, ul, ur)) lanes::roe<float>(F, le, ul, ur);
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    fy[f] = zeroY ? 0.f : F[yFrameOf(f)];
                    fyp[(warp * 5 + f) * 32 + lane] = fy[f];
                }
            }
            float fx[5], fz[5];
            if (tileRow) {
                // x and z half slopes of the cell, after the y face (fewer
                // values live across it), on register pairs in the interface
                // frames (pair j: global field j on the x axis, field
                // zGlobalOf(j) on the z axis)
                float2 Lxz[5], Rxz[5];
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    int const g = zGlobalOf(j);
                    float2 const c = make_float2(p0[j * FS], p0[g * FS]);
                    float2 const dL = lanes::sub(c, make_float2(p0[j * FS - 1], pm[g * FS]));
                    float2 const dR = lanes::sub(make_float2(p0[j * FS + 1], pp[g * FS]), c);
                    float2 const h = lanes::halfSlope<SLOPE>(dL, dR, slim);
                    Lxz[j] = lanes::sub(c, h);
                    Rxz[j] = lanes::add(c, h);
                }
                // the left x face (left lane's R | own L) and the lower z face
                // (the cell below's R | own L), on register pairs
                lanes::C5<float2> UL, UR;
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    UL.u[j] = make_float2(__shfl_up_sync(FULL, Rxz[j].x, 1), Rz[j]);
                    UR.u[j] = Lxz[j];
                    Rz[j] = Rxz[j].y;   // the next plane's cell below
                }
                if (iz >= 2) {
                    float2 F[5];
                    bool const plain = lanes::roeUp2(F, le, UL, UR);
                    if (!__all_sync(FULL, plain)) {
                        // a lane has a vacuum side or a degenerate average: every
                        // lane evaluates both faces in the scalar form
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
#pragma unroll
                    for (int f = 0; f < 5; ++f) {
                        fx[f] = zeroX ? 0.f : F[f].x;
                        fz[f] = zeroZ ? 0.f : F[zFrameOf(f)].y;
                    }
                }
            }
            // the y face fluxes are published; a timed-out wait stops the CTA
            if (__syncthreads_or(!ok)) {
                timedOut = true;
                break;
            }
            // plane iz - 2's buffer is free (every thread is past step iz - 1)
            if (iz >= 2 && iz - 2 + NB < nplanes) {
                if (threadIdx.x == 0) issue(iz - 2 + NB);
                ++issued;
            }
            if (iz >= 2 && tileRow) {
                // calcDerivFromFlux: the z difference finishes the cell below
                // (its x and y differences carried), then the x and y
                // differences of this plane's cell, each fma(FL - FR, area,
                // deriv) rounded as written
                float deriv[5];
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    float const fxr = __shfl_down_sync(FULL, fx[f], 1);
                    float const fyl = fyp[((warp - 1) * 5 + f) * 32 + lane];
                    deriv[f] = skipZ ? Dxy[f] : __fmaf_rn(__fsub_rn(Fzp[f], fz[f]), arz, Dxy[f]);
                    float const dx = skipX ? 0.f : __fmaf_rn(__fsub_rn(fx[f], fxr), arx, 0.f);
                    Dxy[f] = skipY ? dx : __fmaf_rn(__fsub_rn(fyl, fy[f]), ary, dx);
                    Fzp[f] = fz[f];
                }
                if (iz >= 3) {
                    // cell (x, yw, zc): u = sum alpha_k u^(k) + sum (beta_k dt) L(u^(k)) + (beta_cur dt) deriv
                    int const zc = z0 - 3 + iz;
                    long long const idx = idx0 + (long long)(iz - 3) * ps;
                    float u[5];
                    if constexpr (EPI == 0) {
                        auto ldAlpha = [&](int m, float* v) {
                            int const b = slotBuf(st.alpha_buf[m], rot, a.rot_buf);
                            if (m == a0) {
#pragma unroll
                                for (int f = 0; f < 5; ++f) v[f] = pre[f];
                            } else if (b == inBuf) {
#pragma unroll
                                for (int f = 0; f < 5; ++f) v[f] = pm[f * FS];
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
                        if (a0 >= 0 && zc + 1 < z0 + planes) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) pre[f] = a0src[f * geo.plane + idx + ps];
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
                        // the stage's structure fixed at compile time: the
                        // same operations as above in the same order
                        if constexpr (EPI == 1) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) u[f] = pm[f * FS];
                        } else if constexpr (EPI == 2) {
#pragma unroll
                            for (int f = 0; f < 5; ++f) u[f] = pre[f];
                        } else {
#pragma unroll
                            for (int f = 0; f < 5; ++f) {
                                float const pb = pm[f * FS];
                                u[f] = lanes::fma(lanes::sub(pre[f], pb), K.calpha[0], pb);
                            }
                        }
                        if constexpr (EPI != 1) {
                            // the next plane's cell (the segment's last plane
                            // read again at its end: no branch), and into L2
                            // eight planes ahead (the last plane repeated near
                            // the end)
                            const float* const pc = a0src + idx;
                            const float* const pn = pc + (zc + 1 < z0 + planes ? ps : 0);
#pragma unroll
                            for (int f = 0; f < 5; ++f) pre[f] = pn[f * geo.plane];
                            int const ahead = zc + 8 < z0 + planes ? 8 : z0 + planes - 1 - zc;
                            const float* const pf = pc + (long long)ahead * ps;
#pragma unroll
                            for (int f = 0; f < 5; ++f)
                                asm volatile("prefetch.global.L2 [%0];" ::"l"(pf + f * geo.plane));
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
                    if (inCols) {
                        if (edgeXY) marchGhosts(out, geo.plane, geo.px, nx, ny, geo.bc, x, yw, idx, u);
                        if (zc < 2 || zc >= nz - 2) marchGhostsZ(out, geo.plane, ps, nz, geo.bc, zc, idx, u);
                    }
                    if (EPI == 2 || st.last) {
                        float const dtc = lanes::dtCell<float, 3>(u, le, K.gdx);
                        if (inCols) dtmin = fast::tmin(dtmin, dtc);
                    }
                }
            }
        }
        if (timedOut) {
            // every copy issued for this item lands (bounded) before the CTA
            // leaves its shared memory
            while (ready < issued) {
                int const b = ready % NB;
                mbar_wait_bounded(&bars[b], (phase >> b) & 1u, kSpinLimit);
                phase ^= 1u << b;
                ++ready;
            }
            return;
        }
        // one FP64 atomicMin per warp and item for the next step's CFL dt
        if ((EPI == 2 || st.last) && tileRow) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dtmin = fast::tmin(dtmin, __shfl_xor_sync(FULL, dtmin, o));
            double const m = (double)dtmin;
            if (lane == 0 && m < __longlong_as_double((long long)kInfBits))
                atomicMin(&ctl->dtmin[ctl->par ^ 1], (unsigned long long)__double_as_longlong(m));
        }
        if (tileRow && __any_sync(FULL, bad) && lane == 0) atomicOr(&ctl->status, DEV_NONFINITE);
    }
}

}  // namespace fz
}  // namespace hc
