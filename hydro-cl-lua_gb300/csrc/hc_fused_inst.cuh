// hc_fused_inst.cuh -- instantiation helpers: each translation unit that
// includes this header compiles a set of stage-kernel configurations and
// registers their launchers.
#pragma once

#include "hc_fused.cuh"
#include "hc_march.cuh"
#include "hc_march3.cuh"

namespace hc {
namespace fz {

// OCC: minimum resident CTAs per SM the kernel is compiled for (0: as many as
// its shared memory and thread count allow).  LANES: lines each thread sweeps
// at once (2: packed FP32 pairs).
// PLM: the reconstruction compiled in (HC_RECON_PLM_CONS / _PRIM / _ATHENA),
// 0 for none ("piecewise constant" included: it is the cell itself), or -1:
// any of the three, read from the scheme at run time.
// FLUX: the fast form's interface flux compiled in (HC_FLUX_*); the exact form
// dispatches at run time and registers as any flux (-1).
template <typename T, int PREC, int DIM, int VAR, int TX, int TY, int TZ, int L, int NT, bool EXACT, int PLM, bool LIM,
          int SLOPE = -1, int UNR = 0, int OCC = 0, int LANES = 1, int FLUX = HC_FLUX_ROE>
void add_stage(std::vector<StageLauncher>& v) {
    using Cfg = StageCfg<T, DIM, TX, TY, TZ, L, NT>;
    constexpr int K = OCC > 0 ? OCC : residentCtas(NT, Cfg::SMEM);
    StageLauncher sl;
    sl.precision = PREC;
    sl.dim = DIM;
    sl.recon = PLM;
    sl.lim = LIM;
    sl.slope = SLOPE;
    sl.variant = VAR;
    sl.tx = TX;
    sl.ty = TY;
    sl.tz = TZ;
    sl.nthreads = NT;
    sl.seg = L;
    sl.unroll = UNR;
    sl.min_ctas = K;
    sl.lanes = LANES;
    sl.flux = EXACT ? -1 : FLUX;
    sl.box[0] = TX + 4;
    sl.box[1] = DIM > 1 ? TY + 4 : 1;
    sl.box[2] = DIM > 2 ? TZ + 4 : 1;
    sl.march = 0;
    sl.smem = Cfg::SMEM;
    sl.launch = [](const StageArgs& a, int slopeLim, int fluxLim, int grid, cudaStream_t s) {
        k_stage<T, DIM, TX, TY, TZ, L, NT, EXACT, PLM, LIM, SLOPE, UNR, K, LANES, FLUX><<<grid, NT, Cfg::SMEM, s>>>(a, slopeLim, fluxLim);
    };
    sl.occupancy = []() -> int {
        auto k = k_stage<T, DIM, TX, TY, TZ, L, NT, EXACT, PLM, LIM, SLOPE, UNR, K, LANES, FLUX>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM) != cudaSuccess) return -1;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NT, Cfg::SMEM) != cudaSuccess) return -1;
        return n;
    };
    v.push_back(sl);
}

// A 2D marching schedule (hc_march.cuh): NW warps per CTA, segments of up
// to H rows, chunks of C rows in NB buffers, the slope limiter SLOPE compiled in
// (-1: read at run time), OCC CTAs per SM.
template <int VAR, int NW, int H, int C, int NB, int SLOPE, int OCC>
void add_march2(std::vector<StageLauncher>& v) {
    using Cfg = MarchCfg<NW, C, NB>;
    StageLauncher sl;
    sl.precision = HC_F32_FUSED;
    sl.dim = 2;
    sl.recon = HC_RECON_PLM_CONS;
    sl.lim = false;
    sl.slope = SLOPE;
    sl.variant = VAR;
    sl.tx = kStripW;
    sl.ty = H;
    sl.tz = 1;
    sl.nthreads = NW * 32;
    sl.seg = H;
    sl.unroll = 1;
    sl.min_ctas = OCC;
    sl.lanes = 1;
    sl.flux = HC_FLUX_ROE;
    sl.box[0] = kMarchBW;
    sl.box[1] = C;
    sl.box[2] = 1;
    sl.march = 1;
    sl.smem = Cfg::SMEM;
    // one kernel per epilogue form; the stage's plan picks it at launch
    sl.launch = [](const StageArgs& a, int slopeLim, int fluxLim, int grid, cudaStream_t s) {
        switch (marchEpi(a.st)) {
        case 1: k_march2<NW, H, C, NB, SLOPE, OCC, 1><<<grid, NW * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        case 2: k_march2<NW, H, C, NB, SLOPE, OCC, 2><<<grid, NW * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        case 3: k_march2<NW, H, C, NB, SLOPE, OCC, 3><<<grid, NW * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        default: k_march2<NW, H, C, NB, SLOPE, OCC, 0><<<grid, NW * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim);
        }
    };
    sl.occupancy = []() -> int {
        void (*ks[4])(StageArgs, int, int) = {k_march2<NW, H, C, NB, SLOPE, OCC, 0>, k_march2<NW, H, C, NB, SLOPE, OCC, 1>,
                                              k_march2<NW, H, C, NB, SLOPE, OCC, 2>, k_march2<NW, H, C, NB, SLOPE, OCC, 3>};
        int occ = 1 << 30;
        for (auto k : ks) {
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM) != cudaSuccess) return -1;
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NW * 32, Cfg::SMEM) != cudaSuccess) return -1;
            occ = n < occ ? n : occ;
        }
        return occ;
    };
    v.push_back(sl);
}

// A 3D marching schedule (hc_march3.cuh): tiles of 30 columns by NWY - 1
// rows (NWY warps per CTA) marching up segments of up to D planes, NB plane buffers,
// the slope limiter SLOPE compiled in (-1: read at run time), OCC CTAs per SM.
template <int VAR, int NWY, int D, int NB, int SLOPE, int OCC>
void add_march3(std::vector<StageLauncher>& v) {
    using Cfg = March3Cfg<NWY, NB>;
    StageLauncher sl;
    sl.precision = HC_F32_FUSED;
    sl.dim = 3;
    sl.recon = HC_RECON_PLM_CONS;
    sl.lim = false;
    sl.slope = SLOPE;
    sl.variant = VAR;
    sl.tx = kStripW;
    sl.ty = NWY - 1;
    sl.tz = D;
    sl.nthreads = NWY * 32;
    sl.seg = D;
    sl.unroll = 1;
    sl.min_ctas = OCC;
    sl.lanes = 1;
    sl.flux = HC_FLUX_ROE;
    sl.box[0] = kMarchBW;
    sl.box[1] = NWY + 3;
    sl.box[2] = 1;
    sl.march = 1;
    sl.smem = Cfg::SMEM;
    sl.launch = [](const StageArgs& a, int slopeLim, int fluxLim, int grid, cudaStream_t s) {
        switch (marchEpi(a.st)) {
        case 1: k_march3<NWY, D, NB, SLOPE, OCC, 1><<<grid, NWY * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        case 2: k_march3<NWY, D, NB, SLOPE, OCC, 2><<<grid, NWY * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        case 3: k_march3<NWY, D, NB, SLOPE, OCC, 3><<<grid, NWY * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim); break;
        default: k_march3<NWY, D, NB, SLOPE, OCC, 0><<<grid, NWY * 32, Cfg::SMEM, s>>>(a, slopeLim, fluxLim);
        }
    };
    sl.occupancy = []() -> int {
        void (*ks[4])(StageArgs, int, int) = {k_march3<NWY, D, NB, SLOPE, OCC, 0>, k_march3<NWY, D, NB, SLOPE, OCC, 1>,
                                              k_march3<NWY, D, NB, SLOPE, OCC, 2>, k_march3<NWY, D, NB, SLOPE, OCC, 3>};
        int occ = 1 << 30;
        for (auto k : ks) {
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM) != cudaSuccess) return -1;
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NWY * 32, Cfg::SMEM) != cudaSuccess) return -1;
            occ = n < occ ? n : occ;
        }
        return occ;
    };
    v.push_back(sl);
}

inline unsigned aux_blocks(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

// The FP32 PLM kernels for the slope limiters the configurations use, plus the
// generic one: minmod, van Leer (comment form), monotized central, superbee.
template <typename T, int PREC, int DIM, int VAR, int TX, int TY, int TZ, int L, int NT, int UNR = 0, int OCC = 0,
          int LANES = 1>
void add_plm_set(std::vector<StageLauncher>& v) {
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, -1, UNR, OCC, LANES>(v);
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, HC_LIMITER_MINMOD, UNR, OCC, LANES>(v);
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, HC_LIMITER_MONOTIZED_CENTRAL, UNR, OCC, LANES>(v);
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, HC_LIMITER_VAN_LEER_ABS, UNR, OCC, LANES>(v);
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, HC_LIMITER_SUPERBEE, UNR, OCC, LANES>(v);
}

// Extra schedules for one compiled-in limiter (the batched configuration's)
// and the generic kernel.
template <typename T, int PREC, int DIM, int VAR, int TX, int TY, int TZ, int L, int NT, int UNR, int OCC = 0, int LANES = 1>
void add_plm_pair(std::vector<StageLauncher>& v) {
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, -1, UNR, OCC, LANES>(v);
    add_stage<T, PREC, DIM, VAR, TX, TY, TZ, L, NT, false, HC_RECON_PLM_CONS, false, HC_LIMITER_VAN_LEER_ABS, UNR, OCC, LANES>(v);
}

// blocks of 256 threads for a grid-stride pass over `cells` cells: one cell
// per thread up to 1024 blocks
inline unsigned gridFor(long long cells) {
    long long const want = (cells + 255) / 256;
    return (unsigned)(want < 1 ? 1 : (want > 1024 ? 1024 : want));
}

template <typename T, int PREC, int DIM, bool EXACT>
void add_aux(std::vector<AuxLauncher>& v) {
    AuxLauncher a;
    a.precision = PREC;
    a.dim = DIM;
    a.fill_ghosts = [](const DevInst* inst, int slot, int buf, cudaStream_t s) {
        k_fill_ghosts<T, DIM><<<1024, 256, 0, s>>>(inst, slot, buf);
        k_extrap_slot<T, DIM><<<64, 256, 0, s>>>(inst, slot, buf);
    };
    a.extrap_stage = [](const DevInst* inst, const DevCtl* ctl, int nslots, int out_buf, int rot_buf, cudaStream_t s) {
        unsigned const gy = (unsigned)(nslots < 65535 ? nslots : 65535);
        k_extrap_stage<T, DIM><<<dim3(8, gy), 256, 0, s>>>(inst, ctl, nslots, out_buf, rot_buf);
    };
    a.constrain = [](const DevInst* inst, int slot, int buf, cudaStream_t s) {
        k_constrain<T, DIM, EXACT><<<1024, 256, 0, s>>>(inst, slot, buf);
    };
    a.calc_dt = [](const DevInst* inst, DevCtl* ctl, int slot, int buf, cudaStream_t s) {
        k_calc_dt<T, DIM, EXACT><<<1024, 256, 0, s>>>(inst, ctl, slot, buf);
    };
    a.xfer = [](const DevInst* inst, int slot, int buf, void* staging, int layout, int dir, long long cells,
                cudaStream_t s) {
        k_xfer<T, DIM><<<gridFor(cells), 256, 0, s>>>(inst, slot, buf, staging, layout, dir);
    };
    a.load = [](const DevInst* inst, DevCtl* ctl, int slot, int buf, const void* staging, int layout, int reset,
                long long cells, cudaStream_t s) {
        k_load_state<T, DIM, EXACT><<<gridFor(cells), 256, 0, s>>>(inst, ctl, slot, buf, staging, layout, reset);
    };
    a.load_many = [](const DevInst* inst, DevCtl* ctl, const XferJobs& J, int layout, int reset, cudaStream_t s) {
        k_load_many<T, DIM, EXACT><<<(unsigned)J.first[J.n], 256, 0, s>>>(inst, ctl, J, layout, reset);
    };
    a.xfer_many = [](const DevInst* inst, const XferJobs& J, int layout, int dir, cudaStream_t s) {
        k_xfer_many<T, DIM><<<(unsigned)J.first[J.n], 256, 0, s>>>(inst, J, layout, dir);
    };
    a.extrap_slot = [](const DevInst* inst, int slot, int buf, cudaStream_t s) {
        k_extrap_slot<T, DIM><<<64, 256, 0, s>>>(inst, slot, buf);
    };
    a.sums = [](const DevInst* inst, int slot, int buf, double vol, double* partial, int blocks, cudaStream_t s) {
        k_sums<T, DIM><<<blocks, 256, 0, s>>>(inst, slot, buf, vol, partial);
    };
    a.fixed_ghosts = [](const DevInst* inst, int slot, int nbufs, cudaStream_t s) {
        k_fixed_ghosts<T, DIM><<<64, 256, 0, s>>>(inst, slot, nbufs);
    };
    a.slab = [](const DevInst* inst, int slot, int buf, int axis, int side, int dir, double* staging, long long cells,
                cudaStream_t s) {
        k_slab<T, DIM><<<gridFor(cells), 256, 0, s>>>(inst, slot, buf, axis, side, dir, staging);
    };
    v.push_back(a);
}

}  // namespace fz
}  // namespace hc
